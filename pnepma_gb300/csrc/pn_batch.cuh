// pn_batch.cuh -- many uneven solves of one P_N order marched together: one launch per sub-step
// covers the active cells of every solve of the group.
//
// Scheduling.  Solves are sorted by their number of energy steps (longest first) and aligned at
// the end of their forward march.  A state is named by j = n_steps - (forward step): j = n_steps
// is the zero initial state, j = 0 the last forward state.  Forward launch t (t = 1..max_steps)
// produces state j = max_steps - t of every solve with n_steps > j; adjoint iteration a uses state
// j = a of every solve with n_steps > a (and the zero state, with the final accumulation, for the
// solves with n_steps == a).  So the solves active in any launch are a prefix of the sorted
// list, and the tile list of each launch is a prefix of one fixed, solve-major tile list.
//
// Checkpoints.  States 0 .. A-1 (the first ones the adjoint needs, the last ones the forward
// produces) are all kept; beyond them, with stride K, state j is kept when (j - A) % K == 0.  The
// adjoint first walks iterations 0 .. A-1 on kept states, then segments [A + mK, A + (m+1)K), each
// after recomputing its states A + mK + 1 .. A + (m+1)K - 1 from state A + (m+1)K (or from the
// zero state).  Because the schedule is aligned in j, every solve checkpoints and recomputes at the
// same launches.  K = 1 keeps every state; A and K are chosen together to recompute the fewest
// steps within the memory budget.
//
// Fused sub-steps (TMA groups).  Sub-step 3 of step j and sub-step 1 of step j - 1 both update the
// odd classes from the even classes of state j, which no launch changes in between; one launch
// runs both on each tile (loads once, updates twice), so a march of n steps takes 2n + 1 launches
// instead of 3n.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <numeric>
#include <type_traits>
#include <string>
#include <vector>

#include "pn_batch_base.h"
#include "pn_solver.cuh"

// Occupancy of the batched kernels: PN_BATCH_MIN_BLOCKS > 0 asks the compiler for at least that
// many resident blocks per SM (fewer registers per thread); PN_BATCH_MAX_TPB caps the tiles one
// block walks.
#ifndef PN_BATCH_MIN_BLOCKS
#define PN_BATCH_MIN_BLOCKS 0
#endif
#ifndef PN_BATCH_MAX_TPB
#define PN_BATCH_MAX_TPB 1
#endif
#if PN_BATCH_MIN_BLOCKS > 0
#define PN_BATCH_BOUNDS __launch_bounds__(BLOCK, PN_BATCH_MIN_BLOCKS)
#else
#define PN_BATCH_BOUNDS __launch_bounds__(BLOCK)
#endif

namespace pn {

template <class T>
struct BInst {
  Geom g[8];
  long long dev_off[8];
  long long slot_elems;
  T* slots;               // [0] zero state, [1 .. n_full] states 0 .. n_full - 1, then the
                          // checkpoints of states n_full, n_full + K, ..., then work slots
  T* lam;
  int n_full;             // states kept in full (the first the adjoint sweep needs)
  int n_ck;
  int ns, ne, nr, N1;
  int act[3];
  int active[8];
  T inv_h[3];
  T dE;
  double dEd, dvol, scale_g;
  const T* rho[8];
  double* rbar[8];
  const double* bmat_f[3][8];
  const double* bmat_a[3][8];
  const double* beam[8];
  double* acs;            // [cell][r] device copies of the inputs
  double* noa;            // [cell][e]
  double* wint;           // [cell][r]
  double* wsum;           // [cell][r] sum over adjoint iterations of coef_r u0 (eee moment 0)
  double* wsrc;           // [cell][r] acs noa ibar_r: the adjoint source weights of one sweep
  double* ibar;           // scaled cotangent [r]
  double* out_mul;        // factor undoing the scaling of the adjoint outputs
  double* I;              // [r] intensities of the last forward
  double* integral;       // [ns + 1][r]
  int xel[MAXR];
  // per-step tables
  const T* fwd_s;         // [ns][ne]
  const T* fwd_c;         // [ns][ne][N1]
  const double* fwd_bc;   // [ns]
  const double* fwd_sigma;   // [ns + 1][r]
  const double* fwd_weight;  // [ns + 1]
  const T* adj_s;         // [ns][ne]
  const T* adj_c;         // [ns][ne][N1]
  const double* adj_src;  // [ns][r]
  const T* int_s;         // [ns + 1][ne]
  const T* int_c;         // [ns + 1][ne][N1]
  const double* int_bc;   // [ns + 1]
  const double* int_coef; // [ns + 1][r]  dE dvol sigma w
  const double* int_wfac; // [ns + 1]     dvol dE w
  double src_mag;         // largest adjoint cross-section x 1e23 (scaling of the cotangent)
  // caller layout of rho / rho_bar
  int shape[8][3];
  long long off_rho[8];
  long long n_rho;
  long long n_eee;
  long long rho_off[8];
  int px[8];
  // work segments per list (0: parity-0 targets, 1: parity-1 targets, 2: all classes)
  int tile0[3];
  int ptile0;             // first slot of this solve's eee tiles in the compact partial arrays
  int n_ptile;            // its eee tiles: the leading tiles of list 0
  int nseg[3];
  Seg seg[3][MAXSEG];
  // boundary blocks in the state precision (rounded once on the host), for the TMA tile kernels'
  // face ghosts; after the segments so that the generic kernels' staged head stays as it is
  const T* bmt_f[3][8];
  const T* bmt_a[3][8];
};

struct BTile {
  int inst;
  int seg;
  int lb;   // block index local to the segment
  int pad;  // partial slot of an eee tile of list 0, else -1
};

enum { BM_FORWARD = 0, BM_RECOMPUTE = 1, BM_ADJOINT = 2 };

template <class T>
struct BLaunch {
  const BInst<T>* inst;
  const BTile* tiles;
  int list;
  int mode;
  int j;        // forward / recompute: state produced; adjoint / integrate: iteration
  int sub;      // 1, 2, 3
  int K;
  double* partial;   // forward even sub-step: [eee tile][pr] of this launch
  int pr;            // line stride of the partials (largest n_r of the group)
  int n_tiles;       // active tiles of this launch
  int tpb;           // consecutive tiles per block
};

// per-block arguments in shared memory, same member names as SubArgs / IntArgs
template <class T, int N>
struct BSub {
  Geom g[8];
  T* rd[8];
  T* wr[8];
  const T* rho[8];
  const double* bmat[3][8];
  const double* beam[8];
  int act[3];
  int ne, nr;
  int adjoint_source;
  T dt;
  double bc, scale_g;
  T s[MAXE];
  T c[MAXE][N + 1];
  const double* wsrc;     // [cell][r] acs noa ibar_r (adjoint source weights)
  int xel[MAXR];
  double sig_src[MAXR];
  static constexpr bool line_src = true;
  const double* wint;
  T inv_h[3];
  T* cache[8];        // unused by the batched kernels (cache_mode 0)
  int cache_mode;
  static constexpr int pre_ghosts = 0;   // face threads form their ghosts
};

template <class T, int N>
struct BInt {
  Geom g[8];
  T* u[8];
  const T* lam[8];
  const T* rho[8];
  double* rbar[8];
  const double* bmat[3][8];
  const double* beam[8];
  int act[3];
  int ne, nr;
  double bc, scale_g, wfac;
  T s[MAXE];
  T c[MAXE][N + 1];
  double* wsum;           // [cell][line] sum over iterations of coef_r u0
  int xel[MAXR];
  double coef[MAXR];
  T inv_h[3];
  static constexpr bool line_sums = true;
  static constexpr int pre_ghosts = 0;   // face threads form their ghosts
};

// Slot of state j: the zero state past the end of the march, a kept state, a checkpoint, or a
// work slot (alternating in the forward sweep; one per state of a recomputed segment).
template <class T>
__device__ __forceinline__ T* bslot(const BInst<T>& I, int j, int K, bool segment) {
  if (j >= I.ns) return I.slots;
  if (j < I.n_full) return I.slots + (long long)(1 + j) * I.slot_elems;
  const int r = j - I.n_full;
  if (r % K == 0) return I.slots + (long long)(1 + I.n_full + r / K) * I.slot_elems;
  const int w = segment ? (r % K - 1) : (j & 1);
  return I.slots + (long long)(1 + I.n_full + I.n_ck + w) * I.slot_elems;
}

// Words of a BInst before its segment tables: what a block stages (the segments are read from
// global memory, one per tile).
template <class T>
constexpr int binst_head_words() {
  return (int)(offsetof(BInst<T>, seg) / 4);
}

// Copy the head of solve `q`'s descriptor into shared memory with every thread of the block
// (coalesced 4-byte words), so the per-block arguments can then be filled in parallel from it.
// Only the fields before `seg` are valid in the returned reference.
template <class T>
__device__ __forceinline__ const BInst<T>& stage_instance(const BInst<T>* inst, int q, unsigned int* raw) {
  constexpr int W = binst_head_words<T>();
  const unsigned int* src = reinterpret_cast<const unsigned int*>(inst + q);
  for (int w = threadIdx.x; w < W; w += BLOCK) raw[w] = src[w];
  __syncthreads();
  return *reinterpret_cast<const BInst<T>*>(raw);
}

// per-block arguments of a sub-step for solve I (threads fill disjoint fields; caller syncs)
template <class T, int N, bool ADJ>
__device__ __forceinline__ void fill_sub(BSub<T, N>& a, const BInst<T>& I, const BLaunch<T>& L) {
  const int par = L.list;
  const int tid = threadIdx.x;
  int row;
  T* own_rd;
  T* own_wr;
  T* from_rd;
  if (!ADJ) {
    const bool segment = L.mode == BM_RECOMPUTE;
    T* src = bslot(I, L.j + 1, L.K, segment);
    T* dst = bslot(I, L.j, L.K, segment);
    own_rd = (L.sub == 3) ? dst : src;
    own_wr = dst;
    from_rd = (L.sub == 1) ? src : dst;
    row = I.ns - L.j - 1;
  } else {
    own_rd = own_wr = from_rd = I.lam;
    row = L.j;
  }
  if (tid < 8) {
    const int c = tid;
    a.g[c] = I.g[c];
    const bool tgt = class_parity_d(c) == par;
    a.rd[c] = I.active[c] ? (tgt ? own_rd : from_rd) + I.dev_off[c] : nullptr;
    a.wr[c] = I.active[c] ? own_wr + I.dev_off[c] : nullptr;
    a.rho[c] = I.rho[c];
    for (int k = 0; k < 3; ++k) a.bmat[k][c] = ADJ ? I.bmat_a[k][c] : I.bmat_f[k][c];
    a.beam[c] = I.beam[c];
  } else if (tid == 8) {
    for (int k = 0; k < 3; ++k) {
      a.act[k] = I.act[k];
      a.inv_h[k] = I.inv_h[k];
    }
    a.ne = I.ne;
    a.nr = I.nr;
    a.dt = L.sub == 2 ? I.dE : I.dE * T(0.5);
    a.scale_g = I.scale_g;
    a.wsrc = I.wsrc;
    a.wint = I.wint;
    a.adjoint_source = ADJ ? 1 : 0;
    a.cache_mode = 0;
    a.bc = ADJ ? 0.0 : I.fwd_bc[row];
    for (int r = 0; r < MAXR; ++r) a.xel[r] = I.xel[r];
  } else if (tid >= 16 && tid < 16 + MAXR) {
    const int r = tid - 16;
    a.sig_src[r] = (ADJ && r < I.nr) ? I.adj_src[(long long)row * I.nr + r] : 0.0;
  } else if (tid >= 24 && tid < 24 + MAXE) {
    const int e = tid - 24;
    a.s[e] = e < I.ne ? (ADJ ? I.adj_s[row * I.ne + e] : I.fwd_s[row * I.ne + e]) : T(0);
  } else if (tid >= 32 && tid < 32 + MAXE * (N + 1)) {
    const int e = (tid - 32) / (N + 1), l = (tid - 32) % (N + 1);
    const T* cc = ADJ ? I.adj_c : I.fwd_c;
    a.c[e][l] = e < I.ne ? cc[((long long)row * I.ne + e) * (N + 1) + l] : T(0);
  }
}

// One block walks L.tpb consecutive tiles of the launch's list; the solve's arguments are staged
// once and again only when the next tile belongs to another solve (tiles are solve-major).
template <class T, int N, bool ADJ, int DIMS>
__global__ void PN_BATCH_BOUNDS batch_substep_kernel(const __grid_constant__ BLaunch<T> L) {
  __shared__ BSub<T, N> a;
  __shared__ __align__(16) unsigned int raw[binst_head_words<T>() + 1];
  __shared__ double red[BLOCK / 32][MAXR];
  const int t_end = min(L.n_tiles, ((int)blockIdx.x + 1) * L.tpb);
  int cur = -1;
  for (int t = (int)blockIdx.x * L.tpb; t < t_end; ++t) {
    const BTile tl = L.tiles[t];
    if (tl.inst != cur) {
      if (cur >= 0) __syncthreads();   // every thread is done with the previous solve's arguments
      const BInst<T>& I0 = stage_instance(L.inst, tl.inst, raw);
      fill_sub<T, N, ADJ>(a, I0, L);
      __syncthreads();
      cur = tl.inst;
    }
    const BInst<T>& I = *reinterpret_cast<const BInst<T>*>(raw);
    Seg one = L.inst[tl.inst].seg[L.list][tl.seg];
    one.block0 = 0;
    int i = 0, j = 0, k = 0, s0;
    const bool ok = locate(&one, 1, tl.lb, threadIdx.x, s0, i, j, k);
    const bool face = one.kind == 1;
    double part[MAXR];
#pragma unroll
    for (int r = 0; r < MAXR; ++r) part[r] = 0.0;
    double* pp = (L.partial != nullptr) ? part : nullptr;
    if (ok) {
      switch (one.cls) {
        case 0: substep_cell<T, N, 0, ADJ, true, BSub<T, N>, DIMS>(a, i, j, k, face, pp); break;
        case 1: substep_cell<T, N, 1, ADJ, true, BSub<T, N>, DIMS>(a, i, j, k, face, pp); break;
        case 2: substep_cell<T, N, 2, ADJ, true, BSub<T, N>, DIMS>(a, i, j, k, face, pp); break;
        case 3: substep_cell<T, N, 3, ADJ, true, BSub<T, N>, DIMS>(a, i, j, k, face, pp); break;
        case 4: substep_cell<T, N, 4, ADJ, true, BSub<T, N>, DIMS>(a, i, j, k, face, pp); break;
        case 5: substep_cell<T, N, 5, ADJ, true, BSub<T, N>, DIMS>(a, i, j, k, face, pp); break;
        case 6: substep_cell<T, N, 6, ADJ, true, BSub<T, N>, DIMS>(a, i, j, k, face, pp); break;
        default: substep_cell<T, N, 7, ADJ, true, BSub<T, N>, DIMS>(a, i, j, k, face, pp); break;
      }
    }
    if (L.partial != nullptr && one.cls == 0) {   // block-uniform: only eee tiles carry intensity
      const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      // only the group's lines: FP64 adds are scarce on this GPU (2 per SM per clock)
#pragma unroll
      for (int r = 0; r < MAXR; ++r) {
        if (r < L.pr) {
          double v = part[r];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
          if (lane == 0) red[w][r] = v;
        }
      }
      __syncthreads();
      if (threadIdx.x < L.pr) {
        double v = 0.0;
#pragma unroll
        for (int q = 0; q < BLOCK / 32; ++q) v += red[q][threadIdx.x];
        L.partial[(long long)tl.pad * L.pr + threadIdx.x] = v;
      }
      __syncthreads();   // red is reused by the next tile
    }
  }
}

template <class T, int N>
__device__ __forceinline__ void fill_int(BInt<T, N>& a, const BInst<T>& I, const BLaunch<T>& L) {
  const int it = L.j;   // iteration; it == ns is the final accumulation on the zero state
  const int tid = threadIdx.x;
  if (tid < 8) {
    const int c = tid;
    T* u = bslot(I, it, L.K, true);
    a.g[c] = I.g[c];
    a.u[c] = I.active[c] ? u + I.dev_off[c] : nullptr;
    a.lam[c] = I.active[c] ? I.lam + I.dev_off[c] : nullptr;
    a.rho[c] = I.rho[c];
    a.rbar[c] = I.rbar[c];
    for (int k = 0; k < 3; ++k) a.bmat[k][c] = I.bmat_f[k][c];
    a.beam[c] = I.beam[c];
  } else if (tid == 8) {
    for (int k = 0; k < 3; ++k) {
      a.act[k] = I.act[k];
      a.inv_h[k] = I.inv_h[k];
    }
    a.ne = I.ne;
    a.nr = I.nr;
    a.bc = I.int_bc[it];
    a.scale_g = I.scale_g;
    a.wfac = I.int_wfac[it];
    a.wsum = I.wsum;
    for (int r = 0; r < MAXR; ++r) a.xel[r] = I.xel[r];
  } else if (tid >= 16 && tid < 16 + MAXR) {
    const int r = tid - 16;
    a.coef[r] = r < I.nr ? I.int_coef[(long long)it * I.nr + r] : 0.0;
  } else if (tid >= 24 && tid < 24 + MAXE) {
    const int e = tid - 24;
    a.s[e] = e < I.ne ? I.int_s[(long long)it * I.ne + e] : T(0);
  } else if (tid >= 32 && tid < 32 + MAXE * (N + 1)) {
    const int e = (tid - 32) / (N + 1), l = (tid - 32) % (N + 1);
    a.c[e][l] = e < I.ne ? I.int_c[((long long)it * I.ne + e) * (N + 1) + l] : T(0);
  }
}

template <class T, int N, int DIMS>
__global__ void PN_BATCH_BOUNDS batch_integrate_kernel(const __grid_constant__ BLaunch<T> L) {
  __shared__ BInt<T, N> a;
  __shared__ __align__(16) unsigned int raw[binst_head_words<T>() + 1];
  const int t_end = min(L.n_tiles, ((int)blockIdx.x + 1) * L.tpb);
  int cur = -1;
  for (int t = (int)blockIdx.x * L.tpb; t < t_end; ++t) {
    const BTile tl = L.tiles[t];
    if (tl.inst != cur) {
      if (cur >= 0) __syncthreads();
      const BInst<T>& I0 = stage_instance(L.inst, tl.inst, raw);
      fill_int<T, N>(a, I0, L);
      __syncthreads();
      cur = tl.inst;
    }
    Seg one = L.inst[tl.inst].seg[2][tl.seg];
    one.block0 = 0;
    int i = 0, j = 0, k = 0, s0;
    if (!locate(&one, 1, tl.lb, threadIdx.x, s0, i, j, k)) continue;
    const bool face = one.kind == 1;
    switch (one.cls) {
      case 0: integrate_cell<T, N, 0, true, BInt<T, N>, DIMS>(a, i, j, k, face); break;
      case 1: integrate_cell<T, N, 1, true, BInt<T, N>, DIMS>(a, i, j, k, face); break;
      case 2: integrate_cell<T, N, 2, true, BInt<T, N>, DIMS>(a, i, j, k, face); break;
      case 3: integrate_cell<T, N, 3, true, BInt<T, N>, DIMS>(a, i, j, k, face); break;
      case 4: integrate_cell<T, N, 4, true, BInt<T, N>, DIMS>(a, i, j, k, face); break;
      case 5: integrate_cell<T, N, 5, true, BInt<T, N>, DIMS>(a, i, j, k, face); break;
      case 6: integrate_cell<T, N, 6, true, BInt<T, N>, DIMS>(a, i, j, k, face); break;
      default: integrate_cell<T, N, 7, true, BInt<T, N>, DIMS>(a, i, j, k, face); break;
    }
  }
}

// ----------------------------------------------------------------------------------------------
// batched helpers: one launch over every solve of the group (blockIdx.y = solve)
// ----------------------------------------------------------------------------------------------


template <class T>
__global__ void batch_load_kernel(const BInst<T>* __restrict__ inst, const BIo* __restrict__ io) {
  const BInst<T>& I = inst[blockIdx.y];
  const BIo& o = io[blockIdx.y];
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  // densities: caller layout [class][point][e] -> device [e][z][y][x] per active class
  for (long long q = t0; q < I.n_rho; q += stride) {
    int c = 0;
    while (c < 7 && q >= I.off_rho[c + 1]) ++c;
    if (!I.active[c]) continue;
    const long long r0 = q - I.off_rho[c];
    const long long p = r0 / I.ne;
    const int e = (int)(r0 - p * I.ne);
    const int nx = I.shape[c][0], ny = I.shape[c][1];
    const int x = (int)(p % nx);
    const long long rest = p / nx;
    const int y = (int)(rest % ny);
    const int z = (int)(rest / ny);
    T* dst = const_cast<T*>(I.rho[c]);
    dst[e * I.g[c].ms + ((long long)z * ny + y) * I.px[c] + x] = T(o.rho[q]);
  }
  for (long long q = t0; q < I.n_eee * I.ne; q += stride) I.noa[q] = o.noa[q];
  for (long long q = t0; q < I.n_eee * I.nr; q += stride) {
    I.acs[q] = o.acs[q];
    const long long cell = q / I.nr;
    const int r = (int)(q - cell * I.nr);
    I.wint[q] = o.acs[q] * o.noa[cell * I.ne + I.xel[r]];
  }
}

template <class T>
__global__ void batch_zero_kernel(const BInst<T>* __restrict__ inst, int which) {
  const BInst<T>& I = inst[blockIdx.y];
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (which == 0) {
    for (long long q = t0; q < I.slot_elems; q += stride) I.slots[q] = T(0);
    for (long long q = t0; q < (long long)(I.ns + 1) * I.nr; q += stride) I.integral[q] = 0.0;
  } else {
    for (long long q = t0; q < I.slot_elems; q += stride) I.lam[q] = T(0);
    for (int c = 0; c < 8; ++c)
      if (I.active[c])
        for (long long q = t0; q < I.g[c].ms * I.ne; q += stride) I.rbar[c][q] = 0.0;
    for (long long q = t0; q < I.n_eee * I.nr; q += stride) I.wsum[q] = 0.0;
  }
}

// integral[i][r] of solve k = sum over its eee tiles of the partials of forward launch t
template <class T>
__global__ void batch_reduce_kernel(const BInst<T>* __restrict__ inst, const double* __restrict__ partial,
                                    int max_ns, int n_ptiles, int pr) {
  const BInst<T>& I = inst[blockIdx.y];
  const int i = blockIdx.x + 1;  // forward step 1..ns
  if (i > I.ns) return;
  const int t = max_ns - I.ns + i;  // launch index (1-based)
  __shared__ double buf[MAXR][128];
  for (int r = 0; r < MAXR; ++r) {
    double v = 0.0;
    if (r < pr)
      for (int b = threadIdx.x; b < I.n_ptile; b += blockDim.x)
        v += partial[((long long)(t - 1) * n_ptiles + I.ptile0 + b) * pr + r];
    buf[r][threadIdx.x] = v;
  }
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int r = 0; r < MAXR; ++r) buf[r][threadIdx.x] += buf[r][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < I.nr) I.integral[(long long)i * I.nr + threadIdx.x] = buf[threadIdx.x][0];
}

template <class T>
__global__ void batch_final_kernel(const BInst<T>* __restrict__ inst) {
  const BInst<T>& I = inst[blockIdx.x];
  const int r = threadIdx.x;
  if (r >= I.nr) return;
  double acc = 0.0;
  for (int i = 0; i <= I.ns; ++i)
    acc = acc + I.dEd * I.dvol * I.fwd_sigma[(long long)i * I.nr + r] * I.integral[(long long)i * I.nr + r] * I.fwd_weight[i];
  I.I[r] = acc / I.scale_g;
}

template <class T>
__global__ void batch_copy_I_kernel(const BInst<T>* __restrict__ inst, const BIo* __restrict__ io) {
  const BInst<T>& I = inst[blockIdx.x];
  if (threadIdx.x < I.nr && io[blockIdx.x].I) io[blockIdx.x].I[threadIdx.x] = I.I[threadIdx.x];
}

template <class T>
__global__ void batch_prep_ibar_kernel(const BInst<T>* __restrict__ inst, const BIo* __restrict__ io, int fp32) {
  const BInst<T>& I = inst[blockIdx.x];
  if (threadIdx.x != 0) return;
  const double* in = io[blockIdx.x].ibar;
  double m = 0.0;
  for (int r = 0; r < I.nr; ++r) m = fmax(m, fabs(in[r]));
  double sc = 1.0;
  const double q = m * I.src_mag;
  if (fp32 && q > 0.0 && isfinite(q)) sc = ldexp(1.0, -(int)llrint(log2(q)));
  for (int r = 0; r < I.nr; ++r) I.ibar[r] = in[r] * sc;
  I.out_mul[0] = 1.0 / (I.scale_g * sc);
}

// adjoint source weights acs(cell, r) noa(cell, e_r) ibar_r of every solve (after the scaled ibar)
template <class T>
__global__ void batch_prep_src_kernel(const BInst<T>* __restrict__ inst) {
  const BInst<T>& I = inst[blockIdx.y];
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < I.n_eee * I.nr; q += stride) {
    const long long ce = q / I.nr;
    const int r = (int)(q - ce * I.nr);
    I.wsrc[q] = I.acs[q] * I.noa[ce * I.ne + I.xel[r]] * I.ibar[r];
  }
}

template <class T>
__global__ void batch_store_kernel(const BInst<T>* __restrict__ inst, const BIo* __restrict__ io) {
  const BInst<T>& I = inst[blockIdx.y];
  const BIo& o = io[blockIdx.y];
  const double mul = I.out_mul[0];
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  for (long long q = t0; q < I.n_rho; q += stride) {
    int c = 0;
    while (c < 7 && q >= I.off_rho[c + 1]) ++c;
    double v = 0.0;
    if (I.active[c]) {
      const long long r0 = q - I.off_rho[c];
      const long long p = r0 / I.ne;
      const int e = (int)(r0 - p * I.ne);
      const int nx = I.shape[c][0], ny = I.shape[c][1];
      const int x = (int)(p % nx);
      const long long rest = p / nx;
      const int y = (int)(rest % ny);
      const int z = (int)(rest / ny);
      v = I.rbar[c][e * I.g[c].ms + ((long long)z * ny + y) * I.px[c] + x] * mul;
    }
    o.rho_bar[q] = v;
  }
  // acs_bar(cell, r) = noa(cell, e_r) ibar_r W_r;  noa_bar(cell, e) = sum over the lines r of
  // element e of acs(cell, r) ibar_r W_r
  for (long long q = t0; q < I.n_eee * I.ne; q += stride) {
    const long long ce = q / I.ne;
    const int e = (int)(q - ce * I.ne);
    double v = 0.0;
    for (int r = 0; r < I.nr; ++r)
      if (I.xel[r] == e) v += I.acs[ce * I.nr + r] * I.wsum[ce * I.nr + r] * I.ibar[r];
    o.noa_bar[q] = v * mul;
  }
  for (long long q = t0; q < I.n_eee * I.nr; q += stride) {
    const long long ce = q / I.nr;
    const int r = (int)(q - ce * I.nr);
    o.acs_bar[q] = I.noa[ce * I.ne + I.xel[r]] * I.wsum[q] * I.ibar[r] * mul;
  }
}

}  // namespace pn

#include "pn_batch_tma.cuh"

namespace pn {

// ----------------------------------------------------------------------------------------------
// host side: one group of solves with the same order and element type
// ----------------------------------------------------------------------------------------------


// A chunk of a call's solve pointers, carried to the device in kernel parameters (at most
// IoChunk::MAX solves per launch; 25.6 KB of parameters).
struct IoChunk {
  static constexpr int MAX = 400;
  BIo* dst;
  int n;
  int pad_;
  BIo v[MAX];
};
static_assert(sizeof(IoChunk) < 32000, "IoChunk must fit the kernel parameter space");

static __global__ void batch_put_io_kernel(const __grid_constant__ IoChunk c) {
  for (int i = threadIdx.x; i < c.n; i += blockDim.x) c.dst[i] = c.v[i];
}

template <class T, int N, int DIMS>
class BatchGroup : public BatchGroupBase {
 public:
  std::vector<Layout> Ls;
  std::vector<int> order;      // position in group -> caller index (sorted by steps, longest first)
  std::vector<BInst<T>> hinst;
  BInst<T>* dinst = nullptr;
  BIo* dio = nullptr;
  std::vector<BTile> tiles[3];
  BTile* dtiles[3] = {nullptr, nullptr, nullptr};
  std::vector<int> tile_end[3];   // cumulative tiles per solve (in group order)
  double* partial = nullptr;
  int n_ptiles = 0, pr = 1;   // compact partials: eee tiles of all solves, line stride
  int max_ns = 0, K = 1, n = 0;
  int A = 0;                   // states 0 .. A-1 kept in full
  long long recomputed = 0;    // forward steps one adjoint recomputes (all solves)
  std::vector<void*> allocs;
  long long bytes = 0;
  cudaGraphExec_t gf = nullptr, ga = nullptr;
  cudaStream_t cap = nullptr;
  long long nl_f = 0, nl_a = 0, nl = 0;
  int sms = 152;
  // FP32 2D (x, y) and 3D groups: every sub-step and density integral through the TMA tile kernels
  bool use_tma = false;
  std::vector<const pn_desc*> cur_descs;   // the group's descriptors while create() runs
  std::vector<double> checked_advection;   // coupling blocks already checked against the stencil
  std::vector<TTile> ttl[3];     // per list: 0 / 1 parity targets, 2 every class (density integral)
  std::vector<int> tend[3];   // per solve: end of its tiles (solve-major lists)
  TTile* dttl[3] = {nullptr, nullptr, nullptr};
  void* dirows = nullptr;
  TSolve* dsolves = nullptr;
  int tma_int_grid = 0;
  CUtensorMap* dmaps = nullptr;
  void* drows = nullptr;
  int* dstatus = nullptr;          // [0] status of the latest calls, [1] test expiries left
  bool test_expire = false;         // PN_BATCH_TEST_EXPIRE_WAIT
  int cta_cap = 0;                  // resident CTAs per SM of the tile kernels (0: occupancy)
  bool parity_tiles = false;        // PN_BATCH_PARITY_TILES
  // one persistent launch per sweep (TMA groups replayed as graphs, see batch_sweep_kernel): the
  // steps of each sweep are planned once before the graphs are captured
  bool sweep = false;
  bool planning = false;            // record() collects the TMA steps only, launching nothing
  std::vector<TStep> rec_steps;
  struct SweepPlan {
    TStep* steps = nullptr;
    int* dep = nullptr;
    int* need = nullptr;
    int n_steps = 0, n_items = 0;
  };
  SweepPlan plans[2];               // forward, adjoint
  int* done_d = nullptr;            // [step][solve] completed tiles, zeroed before every sweep
  int sweep_grid = 0;
  int tma_grid[2] = {0, 0};        // persistent CTAs of the forward / adjoint TMA kernel
  // 2D groups update both target classes of a parity per tile (pn_batch_par.cuh)
  static constexpr bool kPar = DIMS == 3 && PPT == 1;
  bool par = false;
  int par_stage = 0;               // shared memory of one parity-tile stage (the group's elements)
  // Creation never waits for the device: tables go up on `up`, whose event the first forward or
  // adjoint waits on in stream order, and the tape / density zeroing is enqueued with the first
  // forward; graphs are captured on `cap`, which has no work of its own.
  cudaStream_t up = nullptr;
  cudaEvent_t ev_up = nullptr;
  // stream the recorded launches go to: `cap` while capturing the graphs, the caller's stream
  // with PN_BATCH_DIRECT_LAUNCH (no graphs: a group run once, as a served wave is, gains nothing
  // from them, and instantiating them can wait on the device)
  cudaStream_t ls = nullptr;
  bool direct = false;
  std::vector<std::pair<void*, size_t>> zero_ranges;
  bool zeroed = false;

  ~BatchGroup() override {
    if (gf) cudaGraphExecDestroy(gf);
    if (ga) cudaGraphExecDestroy(ga);
    if (up) {
      // arena ranges are reused at once: let uploads still in flight land first
      if (arena) cudaStreamSynchronize(up);
      cudaStreamDestroy(up);
    }
    if (ev_up) cudaEventDestroy(ev_up);
    if (cap) cudaStreamDestroy(cap);
    for (void* p : allocs) {
      if (arena) arena->free(p);
      else cudaFree(p);
    }
  }
  long long device_bytes() const override { return bytes; }
  // the recorded launches plus the call's own: the pointer upload, load / prep and store kernels
  long long launches_forward() const override { return nl_f + 2 + (n + IoChunk::MAX - 1) / IoChunk::MAX; }
  long long launches_adjoint() const override { return nl_a + 3 + (n + IoChunk::MAX - 1) / IoChunk::MAX; }
  int stride() const override { return K; }
  long long recomputed_steps() const override { return recomputed; }
  bool tma() const override { return use_tma; }
  int device_status() override {
    if (!dstatus) return PN_OK;
    int v = 0;
    PN_CUDA(cudaMemcpy(&v, dstatus, sizeof(int), cudaMemcpyDeviceToHost));
    return v;
  }
  int wait_created() override {
    PN_CUDA(cudaGetLastError());   // launch-time errors only: creation enqueues, it does not wait
    return PN_OK;
  }

  template <class U>
  int alloc(U*& p, long long cnt) {
    void* q = nullptr;
    size_t b = (size_t)std::max<long long>(cnt, 1) * sizeof(U);
    if (arena) {
      q = arena->alloc(b);
      if (!q) {
        err = "no free range of " + std::to_string(b) + " bytes in the memory budget";
        return PN_ERR_NO_MEMORY;
      }
    } else {
      cudaError_t e = cudaMalloc(&q, b);
      if (e != cudaSuccess) {
        cudaGetLastError();
        err = "device allocation of " + std::to_string(b) + " bytes failed: " + cudaGetErrorString(e);
        return PN_ERR_NO_MEMORY;
      }
    }
    allocs.push_back(q);
    bytes += (long long)b;
    p = (U*)q;
    return PN_OK;
  }

  // Small per-solve tables: bump-allocated from device chunks whose bytes are mirrored on the
  // host and copied with one transfer per chunk when the group is complete (flush_staged), so a
  // wave of hundreds of solves does not cost thousands of small transfers.
  struct StageChunk {
    char* dev;
    std::vector<char> host;
    size_t cap;
  };
  std::vector<StageChunk> stage_chunks;

  template <class U>
  int stage(U*& dst, const std::vector<U>& v) {
    const size_t b = ((std::max<size_t>(v.size(), 1) * sizeof(U)) + 255) & ~(size_t)255;
    if (stage_chunks.empty() || stage_chunks.back().host.size() + b > stage_chunks.back().cap) {
      // chunks double from 64 KiB to 16 MiB: small groups stay small, large ones take few copies
      const size_t prev = stage_chunks.empty() ? ((size_t)32 << 10) : stage_chunks.back().cap;
      const size_t cap = std::max<size_t>(b, std::min<size_t>(2 * prev, (size_t)16 << 20));
      char* d = nullptr;
      int rc = alloc(d, (long long)cap);
      if (rc) return rc;
      stage_chunks.push_back(StageChunk{d, {}, cap});
      stage_chunks.back().host.reserve(cap);
    }
    StageChunk& c = stage_chunks.back();
    const size_t off = c.host.size();
    c.host.resize(off + b, 0);
    if (!v.empty()) std::memcpy(c.host.data() + off, v.data(), v.size() * sizeof(U));
    dst = reinterpret_cast<U*>(c.dev + off);
    return PN_OK;
  }

  int flush_staged() {
    for (StageChunk& c : stage_chunks) {
      // pageable source: the call returns once the bytes are staged, so the mirror may go
      if (!c.host.empty()) PN_CUDA(cudaMemcpyAsync(c.dev, c.host.data(), c.host.size(), cudaMemcpyHostToDevice, up));
      std::vector<char>().swap(c.host);
    }
    stage_chunks.clear();
    return PN_OK;
  }

  template <class U>
  int upload(U*& dst, const std::vector<U>& v) {
    int rc = alloc(dst, (long long)v.size());
    if (rc) return rc;
    // pageable source: the call returns once the data is staged, so temporaries may be passed
    if (!v.empty()) PN_CUDA(cudaMemcpyAsync(dst, v.data(), sizeof(U) * v.size(), cudaMemcpyHostToDevice, up));
    return PN_OK;
  }

  int tiles_active(int list, int x) const {
    // tiles of the solves with n_steps > x (a prefix of the group order)
    int cnt = 0;
    for (int q = 0; q < n; ++q)
      if (hinst[q].ns > x) cnt = tile_end[list][q];
    return cnt;
  }

  // checkpoints of the states a .. ns - 1 beyond a kept head of a states
  static int n_ck_for(int ns, int K, int a) { return ns > a ? (ns - a - 1) / K + 1 : 0; }

  // tiles per block: enough blocks to fill the GPU about twice (SMs x 5 resident blocks), at
  // most PN_BATCH_MAX_TPB tiles each
  int tiles_per_block(int nt) const {
    const int target = 2 * sms * 5;
    return std::max(1, std::min(PN_BATCH_MAX_TPB, nt / std::max(1, target)));
  }
  static int n_work_for(int K) { return std::max(2, K - 1); }

  int create(const pn_desc* const* d, const int* idx, int cnt, long long budget, int Kreq, int flags) override {
    n = cnt;
    members.assign(idx, idx + cnt);
    order.resize(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return d[idx[a]]->n_steps > d[idx[b]]->n_steps; });
    std::vector<int> sorted_members(n);
    for (int q = 0; q < n; ++q) sorted_members[q] = idx[order[q]];
    members = sorted_members;
    Ls.resize(n);
    long long slot_total = 0, fixed = 0;
    for (int q = 0; q < n; ++q) {
      const pn_desc* dq = d[members[q]];
      int rc = Ls[q].init(dq, err);
      if (rc) return rc;
      if (Ls[q].ne > MAXE || Ls[q].nr > MAXR || Ls[q].nr < 1) { err = "1..8 x-ray lines and at most 4 elements per solve"; return PN_ERR_UNSUPPORTED; }
      max_ns = std::max(max_ns, Ls[q].ns);
      slot_total += Ls[q].slot_elems * (long long)sizeof(T);
      (void)fixed;
    }
    // tape: the stride K and kept head A that recompute the fewest state values within the budget
    // (K = 1 when every state fits); an explicit stride keeps no head
    auto need = [&](int k, int a) {
      long long b = 0;
      for (int q = 0; q < n; ++q)
        b += (long long)(1 + std::min(a, Ls[q].ns) + n_ck_for(Ls[q].ns, k, a) + n_work_for(k) + 1) *
             Ls[q].slot_elems * (long long)sizeof(T);
      return b;
    };
    auto cost = [&](int k, int a) {   // recomputed state values
      long long c = 0;
      for (int q = 0; q < n; ++q)
        if (Ls[q].ns > a) c += (long long)(Ls[q].ns - a - n_ck_for(Ls[q].ns, k, a)) * Ls[q].slot_elems;
      return c;
    };
    if (Kreq > 0) {
      K = std::min(Kreq, std::max(1, max_ns));
      A = 0;
    } else if (need(1, 0) <= budget) {
      K = 1;
      A = 0;
    } else {
      long long best = -1;
      for (int k = 2; k <= std::max(2, max_ns); ++k) {
        if (need(k, 0) > budget) continue;
        int lo = 0, hi = max_ns;   // largest a with need(k, a) <= budget (need grows with a)
        while (lo < hi) {
          const int mid = (lo + hi + 1) / 2;
          if (need(k, mid) <= budget) lo = mid;
          else hi = mid - 1;
        }
        const long long c = cost(k, lo);
        if (best < 0 || c < best) {
          best = c;
          K = k;
          A = lo;
        }
      }
      if (best < 0) { err = "the batch does not fit the memory budget"; return PN_ERR_NO_MEMORY; }
    }
    recomputed = 0;
    for (int q = 0; q < n; ++q)
      if (Ls[q].ns > A) recomputed += Ls[q].ns - A - n_ck_for(Ls[q].ns, K, A);
    hinst.assign(n, BInst<T>());
    cur_descs.assign(n, nullptr);
    for (int q = 0; q < n; ++q) cur_descs[q] = d[members[q]];
    int rc;
    PN_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    PN_CUDA(cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking));
    PN_CUDA(cudaEventCreateWithFlags(&ev_up, cudaEventDisableTiming));
    {
      int dev = 0;
      PN_CUDA(cudaGetDevice(&dev));
      PN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    }
    // PN_TRACE set in the environment: host time of each phase of the group's creation on stderr
    const bool trace = std::getenv("PN_TRACE") != nullptr;
    auto clk = [] { return std::chrono::steady_clock::now(); };
    auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
      return std::chrono::duration<double, std::milli>(b - a).count();
    };
    const auto t0 = clk();
    for (int q = 0; q < n; ++q) {
      std::memset(&hinst[q], 0, sizeof(BInst<T>));
      if ((rc = build_instance(q, d[members[q]]))) return rc;
    }
    const auto t1 = clk();
    // partial slots: the eee tiles of list 0, numbered per solve in tile order
    n_ptiles = 0;
    pr = 1;
    for (int q = 0; q < n; ++q) {
      int cnt0 = 0;
      for (int sgi = 0; sgi < hinst[q].nseg[0]; ++sgi)
        if (hinst[q].seg[0][sgi].cls == 0) cnt0 += hinst[q].seg[0][sgi].nblocks;
      hinst[q].ptile0 = n_ptiles;
      hinst[q].n_ptile = cnt0;
      n_ptiles += cnt0;
      pr = std::max(pr, hinst[q].nr);
    }
    // tile lists (solve-major, group order)
    for (int list = 0; list < 3; ++list) {
      tile_end[list].assign(n, 0);
      for (int q = 0; q < n; ++q) {
        hinst[q].tile0[list] = (int)tiles[list].size();
        for (int sgi = 0; sgi < hinst[q].nseg[list]; ++sgi) {
          const Seg& sg = hinst[q].seg[list][sgi];
          for (int lb = 0; lb < sg.nblocks; ++lb) tiles[list].push_back(BTile{q, sgi, lb, pslot_of_tile(q, list, sgi, lb)});
        }
        tile_end[list][q] = (int)tiles[list].size();
      }
      if ((rc = upload(dtiles[list], tiles[list]))) return rc;
    }
    if constexpr (std::is_same<T, float>::value && (DIMS == 3 || DIMS == 7)) {
      test_expire = (flags & PN_BATCH_TEST_EXPIRE_WAIT) != 0;
      cta_cap = (flags >> PN_BATCH_CTAS_PER_SM_SHIFT) & 15;
      parity_tiles = (flags & PN_BATCH_PARITY_TILES) != 0;
      if (!(flags & PN_BATCH_GENERIC_KERNELS))
        if ((rc = build_tma())) return rc;
    } else {
      (void)flags;
    }
    const auto t2 = clk();
    if ((rc = flush_staged())) return rc;
    if ((rc = upload(dinst, hinst))) return rc;
    if ((rc = alloc(dio, n))) return rc;
    if ((rc = alloc(partial, (long long)max_ns * std::max(n_ptiles, 1) * pr))) return rc;
    PN_CUDA(cudaEventRecord(ev_up, up));
    const auto t3 = clk();
    direct = (flags & PN_BATCH_DIRECT_LAUNCH) != 0;
    if (!direct && use_tma && (flags & PN_BATCH_SWEEP_LAUNCH)) {
      if ((rc = plan_sweeps())) return rc;
      PN_CUDA(cudaEventRecord(ev_up, up));   // the plans' uploads
    }
    if (!direct) {
      if ((rc = capture(gf, true))) return rc;
      if ((rc = capture(ga, false))) return rc;
      // upload both graphs now, on the idle upload stream: left to its first launch, the adjoint
      // graph's upload queued behind the forward on the caller's stream and held the adjoint call
      // on the host until the forward had finished on the device
      PN_CUDA(cudaGraphUpload(gf, up));
      PN_CUDA(cudaGraphUpload(ga, up));
      PN_CUDA(cudaEventRecord(ev_up, up));
    } else {
      // count the launches of one sweep without issuing them
      nl = 0;
      nl_f = nl_a = 0;
    }
    if (trace) {
      const auto t4 = clk();
      std::fprintf(stderr, "[pn] group N=%d dims=%d solves=%d tma=%d: instances %.1f ms, lists+maps %.1f ms, "
                   "uploads %.1f ms, graphs %.1f ms (%lld + %lld launches)\n",
                   N, DIMS, n, use_tma ? 1 : 0, ms(t0, t1), ms(t1, t2), ms(t2, t3), ms(t3, t4), nl_f, nl_a);
    }
    return PN_OK;
  }

  // TMA path of an FP32 2D (x, y) or 3D group: tile lists, tensor maps, coefficient rows.  Leaves
  // use_tma false (generic kernels) when a class grid is narrower than a box or the driver lacks
  // the tensor-map encoder.
  int build_tma() {
    if constexpr (std::is_same<T, float>::value && (DIMS == 3 || DIMS == 7)) {
      using LY = TmaLayout<N, DIMS>;
      using LI = TmaIntLayout<N, DIMS>;
      if (!encode_tiled_fn()) return PN_OK;
      for (int q = 0; q < n; ++q)
        for (int c = 0; c < 8; ++c)
          // boxes may overhang a narrow grid (the overhang reads zeros); the encoder rejects what
          // the tensor unit cannot address, and the group then keeps the generic kernels
          if (hinst[q].active[c] && (hinst[q].shape[c][0] < 8 || hinst[q].shape[c][1] < 4 || hinst[q].shape[c][0] > 2040 ||
                                     hinst[q].shape[c][1] > 2040))
            return PN_OK;
      int smem_optin = 0, dev = 0;
      PN_CUDA(cudaGetDevice(&dev));
      PN_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
      if (LY::SMEM + 2048 > smem_optin) return PN_OK;
      if (LI::SMEM + 2048 > smem_optin) return PN_OK;
      PN_CUDA(cudaFuncSetAttribute(batch_tma_kernel<N, false, DIMS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   LY::SMEM));
      PN_CUDA(cudaFuncSetAttribute(batch_tma_kernel<N, true, DIMS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   LY::SMEM));
      PN_CUDA(cudaFuncSetAttribute(batch_tma_int_kernel<N, DIMS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   LI::SMEM));
      int occ_i = 0;
      PN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_i, batch_tma_int_kernel<N, DIMS>, NTS, LI::SMEM));
      if (occ_i < 1) return PN_OK;
      tma_int_grid = occ_i * sms;
      int occ_f = 0, occ_a = 0;
      PN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_f, batch_tma_kernel<N, false, DIMS>, NTS, LY::SMEM));
      PN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_a, batch_tma_kernel<N, true, DIMS>, NTS, LY::SMEM));
      par = false;
      if constexpr (kPar) {
        int ne_max = 1;
        for (int q = 0; q < n; ++q) ne_max = std::max(ne_max, hinst[q].ne);
        par_stage = (ParLayout<N>::smem(ne_max) + 127) / 128 * 128;
        if (par_stage + 2048 <= smem_optin && parity_tiles) {
          PN_CUDA(cudaFuncSetAttribute(batch_par_kernel<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       par_stage));
          PN_CUDA(cudaFuncSetAttribute(batch_par_kernel<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       par_stage));
          int pf = 0, pa = 0;
          PN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pf, batch_par_kernel<N, false>, TB, par_stage));
          PN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pa, batch_par_kernel<N, true>, TB, par_stage));
          if (pf >= 1 && pa >= 1) {
            par = true;
            occ_f = pf;
            occ_a = pa;
          }
        }
      }
      if (occ_f < 1 || occ_a < 1) return PN_OK;
      if (cta_cap > 0) {
        occ_f = std::min(occ_f, cta_cap);
        occ_a = std::min(occ_a, cta_cap);
        occ_i = std::min(occ_i, cta_cap);
        tma_int_grid = occ_i * sms;
      }
      tma_grid[0] = occ_f * sms;
      tma_grid[1] = occ_a * sms;
      // coefficient rows: forward then adjoint, per solve
      std::vector<ArgRow<N>> rows;
      std::vector<int> arg_fwd(n), arg_adj(n);
      for (int q = 0; q < n; ++q) {
        const pn_desc* d = cur_descs[q];
        const int ns = hinst[q].ns, ne = hinst[q].ne, nr = hinst[q].nr;
        for (int pass = 0; pass < 2; ++pass) {
          (pass == 0 ? arg_fwd : arg_adj)[q] = (int)rows.size();
          const double* S = pass == 0 ? d->fwd_s : d->adj_s;
          const double* Cc = pass == 0 ? d->fwd_c : d->adj_c;
          for (int row = 0; row < ns; ++row) {
            ArgRow<N> a;
            std::memset(&a, 0, sizeof(a));
            for (int e = 0; e < ne; ++e) {
              a.s[e] = float(S[(long long)row * ne + e]);
              for (int l = 0; l <= N; ++l) a.c[e][l] = float(Cc[((long long)row * ne + e) * (N + 1) + l]);
            }
            if (pass == 0) a.bc = d->fwd_bc[row];
            else
              for (int r = 0; r < nr; ++r) a.sig[r] = d->adj_src_sigma[(long long)row * nr + r];
            rows.push_back(a);
          }
        }
      }
      ArgRow<N>* dr = nullptr;
      int rc;
      if ((rc = upload(dr, rows))) return rc;
      drows = dr;
      // density-integral rows: iterations 0 .. n_steps per solve
      std::vector<IntRow<N>> irows;
      std::vector<int> arg_int(n);
      for (int q = 0; q < n; ++q) {
        const pn_desc* d = cur_descs[q];
        const int ns = hinst[q].ns, ne = hinst[q].ne, nr = hinst[q].nr;
        arg_int[q] = (int)irows.size();
        for (int it = 0; it <= ns; ++it) {
          IntRow<N> a;
          std::memset(&a, 0, sizeof(a));
          for (int e = 0; e < ne; ++e) {
            a.s[e] = float(d->adj_int_s[(long long)it * ne + e]);
            for (int l = 0; l <= N; ++l) a.c[e][l] = float(d->adj_int_c[((long long)it * ne + e) * (N + 1) + l]);
          }
          for (int r = 0; r < nr; ++r)
            a.coef[r] = d->delta_e * d->dvol * d->adj_sigma[(long long)it * nr + r] * d->adj_weight[it];
          a.wfac = d->dvol * d->delta_e * d->adj_weight[it];
          a.bc = d->adj_int_bc[it];
          irows.push_back(a);
        }
      }
      IntRow<N>* dir = nullptr;
      if ((rc = upload(dir, irows))) return rc;
      dirows = dir;
      // tensor maps
      std::vector<CUtensorMap> maps((size_t)n * 8 * TM_KINDS);
      std::memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
      for (int q = 0; q < n; ++q) {
        const BInst<T>& I = hinst[q];
        const long long nslots = 1 + I.n_full + I.n_ck + n_work_for(K);
        for (int c = 0; c < 8; ++c) {
          const int nm = I.g[c].nm;
          if (!I.active[c] || nm == 0) continue;
          CUtensorMap* m = &maps[((size_t)q * 8 + c) * TM_KINDS];
          // (x, y, z, moment, slot); a 2D grid has z extent 1
          const long long st_dims[5] = {I.shape[c][0], I.shape[c][1], I.shape[c][2], nm, nslots};
          const long long st_str[5] = {1, I.px[c], (long long)I.px[c] * I.shape[c][1], I.g[c].ms, I.slot_elems};
          const int boxt[5] = {TX, TY, 1, nm, 1}, boxx[5] = {BW, TY, 1, nm, 1}, boxy[5] = {TX, TY + 1, 1, nm, 1};
          const int boxz[5] = {TX, TY, 2, nm, 1};
          bool ok = encode_f32(&m[TM_ST_T], I.slots + I.dev_off[c], 5, st_dims, st_str, boxt) &&
                    encode_f32(&m[TM_ST_X], I.slots + I.dev_off[c], 5, st_dims, st_str, boxx) &&
                    encode_f32(&m[TM_ST_Y], I.slots + I.dev_off[c], 5, st_dims, st_str, boxy) &&
                    encode_f32(&m[TM_LAM_T], I.lam + I.dev_off[c], 4, st_dims, st_str, boxt) &&
                    encode_f32(&m[TM_LAM_X], I.lam + I.dev_off[c], 4, st_dims, st_str, boxx) &&
                    encode_f32(&m[TM_LAM_Y], I.lam + I.dev_off[c], 4, st_dims, st_str, boxy);
          if (DIMS == 7)
            ok = ok && encode_f32(&m[TM_ST_Z], I.slots + I.dev_off[c], 5, st_dims, st_str, boxz) &&
                 encode_f32(&m[TM_LAM_Z], I.lam + I.dev_off[c], 4, st_dims, st_str, boxz);
          if (par) {
            const int boxn[5] = {NBW, NBH, 1, nm, 1};
            ok = ok && encode_f32(&m[TM_ST_N], I.slots + I.dev_off[c], 5, st_dims, st_str, boxn) &&
                 encode_f32(&m[TM_LAM_N], I.lam + I.dev_off[c], 4, st_dims, st_str, boxn);
          }
          const long long rho_dims[4] = {I.shape[c][0], I.shape[c][1], I.shape[c][2], I.ne};
          const int boxr[4] = {TX, TY, 1, I.ne};
          ok = ok && encode_f32(&m[TM_RHO], const_cast<T*>(I.rho[c]), 4, rho_dims, st_str, boxr);
          ok = ok && encode_tensor(&m[TM_RBAR], I.rbar[c], 4, rho_dims, st_str, boxr, 8);
          if (!ok) return PN_OK;   // generic kernels for this group
        }
      }
      if ((rc = upload(dmaps, maps))) return rc;
      // per-solve arguments staged with every tile
      std::vector<TSolve> hs(n);
      for (int q = 0; q < n; ++q) {
        const BInst<T>& I = hinst[q];
        TSolve& S = hs[q];
        std::memset(&S, 0, sizeof(S));
        S.slots = I.slots;
        S.lam = I.lam;
        S.slot_elems = I.slot_elems;
        S.wint = I.wint;
        S.wsrc = I.wsrc;
        S.wsum = I.wsum;
        for (int c = 0; c < 8; ++c) {
          S.rbar[c] = I.rbar[c];
          S.dev_off[c] = I.dev_off[c];
          S.ms[c] = I.g[c].ms;
          S.px[c] = I.g[c].px;
          S.n0[c] = I.g[c].n[0];
          S.n1[c] = I.g[c].n[1];
          S.n2[c] = I.g[c].n[2];
        }
        for (int r = 0; r < MAXR; ++r) S.xel[r] = I.xel[r];
        for (int k = 0; k < 3; ++k) S.inv_h[k] = I.inv_h[k];
        S.dE = I.dE;
        S.nr = I.nr;
        S.ne = I.ne;
        S.scale_g = I.scale_g;
      }
      if ((rc = upload(dsolves, hs))) return rc;
      if ((rc = alloc(dstatus, 2))) return rc;
      {
        // pageable source: staged before the call returns
        const int st0[2] = {0, test_expire ? 1 : 0};
        PN_CUDA(cudaMemcpyAsync(dstatus, st0, sizeof(st0), cudaMemcpyHostToDevice, up));
      }
      // tiles over every target cell per list; partial slots are the eee tiles of list 0 in tile order
      n_ptiles = 0;
      for (int q = 0; q < n; ++q) {
        hinst[q].ptile0 = 0;
        hinst[q].n_ptile = 0;
      }
      for (int list = 0; list < 3; ++list) {
        tend[list].assign(n, 0);
        for (int q = 0; q < n; ++q) {
          const BInst<T>& I = hinst[q];
          if (list == 0) hinst[q].ptile0 = n_ptiles;
          if (par && list < 2) {
            // parity tiles: every 32 x 4 position of the grid, both targets of the parity
            const int A = par_a(list), B = par_b(list);
            auto ext_of = [&](int c, int x0, int y0) {
              if (!I.active[c] || class_moments_host(c) == 0) return 0;
              const int lox = class_bit(c, 0) ? 1 : 0, hix = class_bit(c, 0) ? I.shape[c][0] - 1 : I.shape[c][0];
              const int loy = class_bit(c, 1) ? 1 : 0, hiy = class_bit(c, 1) ? I.shape[c][1] - 1 : I.shape[c][1];
              const int xv0 = std::max(lox - x0, 0), xv1 = std::min(hix - x0, TX);
              const int yv0 = std::max(loy - y0, 0), yv1 = std::min(hiy - y0, TY);
              return (xv1 > xv0 && yv1 > yv0) ? par_ext(xv0, xv1, yv0, yv1) : 0;
            };
            const int ny = I.shape[0][1], nx = I.shape[0][0];   // the eee grid covers both targets' cells
            for (int y0 = 0; y0 < ny; y0 += TY)
              for (int x0 = 0; x0 < nx; x0 += TX) {
                const int ea = ext_of(A, x0, y0), eb = ext_of(B, x0, y0);
                if (!ea && !eb) continue;
                TTile tt;
                std::memset(&tt, 0, sizeof(tt));
                tt.inst = q;
                tt.cls = list;   // the parity
                tt.x0 = x0;
                tt.y0 = y0;
                tt.ext = ea;
                tt.pad_[0] = eb;
                tt.pslot = (list == 0 && ea) ? n_ptiles++ : -1;
                tt.ns = I.ns;
                tt.n_ck = I.n_ck;
                tt.n_full = I.n_full;
                tt.ne = I.ne;
                tt.arg_fwd = arg_fwd[q];
                tt.arg_adj = arg_adj[q];
                tt.arg_int = arg_int[q];
                tt.z = 0;
                ttl[list].push_back(tt);
              }
            if (list == 0) hinst[q].n_ptile = n_ptiles - hinst[q].ptile0;
            tend[list][q] = (int)ttl[list].size();
            continue;
          }
          for (int c = 0; c < 8; ++c) {
            if (!I.active[c] || (list < 2 && class_parity(c) != list) || class_moments_host(c) == 0) continue;
            int lo3[3], hi3[3];
            for (int k = 0; k < 3; ++k) {
              const int nn = I.shape[c][k];
              lo3[k] = class_bit(c, k) ? 1 : 0;
              hi3[k] = class_bit(c, k) ? nn - 1 : nn;
            }
            // x0 = 32 bx over the class's points; target lanes [lo - x0, hi - x0) within the tile
            for (int z = lo3[2]; z < hi3[2]; ++z)
            for (int y0 = lo3[1]; y0 < hi3[1]; y0 += TY)
              for (int x0 = 0; x0 < hi3[0]; x0 += TX) {
                const int xv0 = std::max(lo3[0] - x0, 0), xv1 = std::min(hi3[0] - x0, TX);
                if (xv1 <= xv0) continue;
                TTile tt;
                std::memset(&tt, 0, sizeof(tt));
                tt.inst = q;
                tt.cls = c;
                tt.x0 = x0;
                tt.y0 = y0;
                tt.ext = xv0 | (xv1 << 8) | (std::min(TY, hi3[1] - y0) << 16);
                tt.pslot = (list == 0 && c == 0) ? n_ptiles++ : -1;
                tt.ns = I.ns;
                tt.n_ck = I.n_ck;
                tt.n_full = I.n_full;
                tt.ne = I.ne;
                tt.arg_fwd = arg_fwd[q];
                tt.arg_adj = arg_adj[q];
                tt.arg_int = arg_int[q];
                tt.z = z;
                ttl[list].push_back(tt);
              }
          }
          if (list == 0) hinst[q].n_ptile = n_ptiles - hinst[q].ptile0;
          tend[list][q] = (int)ttl[list].size();
        }
        if ((rc = upload(dttl[list], ttl[list]))) return rc;
      }
      use_tma = true;
    }
    return PN_OK;
  }

  static int class_moments_host(int c) {
    switch (c) {
      case 0: return Ord<N>::n(0);
      case 1: return Ord<N>::n(1);
      case 2: return Ord<N>::n(2);
      case 3: return Ord<N>::n(3);
      case 4: return Ord<N>::n(4);
      case 5: return Ord<N>::n(5);
      case 6: return Ord<N>::n(6);
      default: return Ord<N>::n(7);
    }
  }

  int pslot_of_tile(int q, int list, int sgi, int lb) const {
    if (list != 0 || hinst[q].seg[0][sgi].cls != 0) return -1;
    int s = hinst[q].ptile0;
    for (int k = 0; k < sgi; ++k)
      if (hinst[q].seg[0][k].cls == 0) s += hinst[q].seg[0][k].nblocks;
    return s + lb;
  }

  static int prefix_active(const std::vector<BInst<T>>& hi, const std::vector<int>& ends, int x) {
    int cnt = 0;
    for (size_t q = 0; q < ends.size(); ++q)
      if (hi[q].ns > x) cnt = ends[q];
    return cnt;
  }

  int build_instance(int q, const pn_desc* d) {
    const Layout& L = Ls[q];
    BInst<T>& I = hinst[q];
    int rc;
    const int ns = L.ns, ne = L.ne, nr = L.nr, N1 = N + 1;
    I.ns = ns; I.ne = ne; I.nr = nr; I.N1 = N1;
    I.slot_elems = L.slot_elems;
    I.n_full = std::min(A, ns);
    I.n_ck = n_ck_for(ns, K, A);
    const int nslots = 1 + I.n_full + I.n_ck + n_work_for(K);
    if ((rc = alloc(I.slots, (long long)nslots * L.slot_elems))) return rc;
    if ((rc = alloc(I.lam, L.slot_elems))) return rc;
    zero_ranges.emplace_back((void*)I.slots, sizeof(T) * (size_t)nslots * L.slot_elems);
    for (int c = 0; c < 8; ++c) {
      I.active[c] = L.active[c];
      I.dev_off[c] = L.dev_off[c];
      if (L.active[c]) {
        for (int k = 0; k < 3; ++k) I.g[c].n[k] = L.shape[c][k];
        I.g[c].px = L.px[c];
        I.g[c].nm = L.nm[c];
        I.g[c].ms = L.ms[c];
      }
      for (int k = 0; k < 3; ++k) I.shape[c][k] = L.shape[c][k];
      I.off_rho[c] = L.off_rho[c];
      I.rho_off[c] = L.rho_off[c];
      I.px[c] = L.px[c];
    }
    I.n_rho = L.n_rho;
    I.n_eee = L.n_eee_cells;
    T* rho_d;
    double* rbar_d;
    if ((rc = alloc(rho_d, L.rho_elems))) return rc;
    if ((rc = alloc(rbar_d, L.rho_elems))) return rc;
    zero_ranges.emplace_back((void*)rho_d, sizeof(T) * (size_t)L.rho_elems);
    for (int c = 0; c < 8; ++c) {
      I.rho[c] = L.active[c] ? rho_d + L.rho_off[c] : nullptr;
      I.rbar[c] = L.active[c] ? rbar_d + L.rho_off[c] : nullptr;
    }
    for (int k = 0; k < 3; ++k) {
      I.act[k] = L.act[k];
      I.inv_h[k] = T(1.0 / d->h[k]);
    }
    I.dE = T(d->delta_e);
    I.dEd = d->delta_e;
    I.dvol = d->dvol;
    // tables
    auto conv = [](const double* p, long long cnt) {
      std::vector<T> v((size_t)cnt);
      for (long long q2 = 0; q2 < cnt; ++q2) v[q2] = T(p[q2]);
      return v;
    };
    auto cpd = [](const double* p, long long cnt) { return std::vector<double>(p, p + cnt); };
    const T* tp;
    const double* dp;
    T* tw;
    double* dw;
    if ((rc = stage(tw, conv(d->fwd_s, (long long)ns * ne)))) return rc; I.fwd_s = tw;
    if ((rc = stage(tw, conv(d->fwd_c, (long long)ns * ne * N1)))) return rc; I.fwd_c = tw;
    if ((rc = stage(dw, cpd(d->fwd_bc, ns)))) return rc; I.fwd_bc = dw;
    if ((rc = stage(dw, cpd(d->fwd_sigma, (long long)(ns + 1) * nr)))) return rc; I.fwd_sigma = dw;
    if ((rc = stage(dw, cpd(d->fwd_weight, ns + 1)))) return rc; I.fwd_weight = dw;
    if ((rc = stage(tw, conv(d->adj_s, (long long)ns * ne)))) return rc; I.adj_s = tw;
    if ((rc = stage(tw, conv(d->adj_c, (long long)ns * ne * N1)))) return rc; I.adj_c = tw;
    if ((rc = stage(dw, cpd(d->adj_src_sigma, (long long)ns * nr)))) return rc; I.adj_src = dw;
    if ((rc = stage(tw, conv(d->adj_int_s, (long long)(ns + 1) * ne)))) return rc; I.int_s = tw;
    if ((rc = stage(tw, conv(d->adj_int_c, (long long)(ns + 1) * ne * N1)))) return rc; I.int_c = tw;
    if ((rc = stage(dw, cpd(d->adj_int_bc, ns + 1)))) return rc; I.int_bc = dw;
    {
      std::vector<double> coef((size_t)(ns + 1) * nr), wf((size_t)(ns + 1));
      for (int j = 0; j <= ns; ++j) {
        wf[j] = d->dvol * d->delta_e * d->adj_weight[j];
        for (int r = 0; r < nr; ++r) coef[(size_t)j * nr + r] = d->delta_e * d->dvol * d->adj_sigma[(long long)j * nr + r] * d->adj_weight[j];
      }
      if ((rc = stage(dw, coef))) return rc; I.int_coef = dw;
      if ((rc = stage(dw, wf))) return rc; I.int_wfac = dw;
    }
    (void)tp;
    (void)dp;
    double smax = 0.0;
    for (long long q2 = 0; q2 < (long long)ns * nr; ++q2) smax = std::max(smax, std::fabs(d->adj_src_sigma[q2]));
    I.src_mag = smax * 1e23;
    for (int r = 0; r < nr; ++r) {
      if (d->xray_element[r] < 0 || d->xray_element[r] >= ne) { err = "xray_element out of range"; return PN_ERR_INVALID; }
      I.xel[r] = d->xray_element[r];
    }
    // coupling: the literal stencil must match the caller's blocks (values as well as sparsity);
    // blocks equal to a set already checked in this group need no second check
    bool coupling_checked = false;
    if (!checked_advection.empty() && (long long)checked_advection.size() == L.n_adv &&
        std::memcmp(checked_advection.data(), d->advection, sizeof(double) * (size_t)L.n_adv) == 0)
      coupling_checked = true;
    if (!coupling_checked) {
      const double* pa = d->advection;
      for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 8; ++c) {
          const int nrow = L.nm[c], ncol = L.nm[class_switch(c, k)];
          const int off = Ord<N>::off(c, k);
          const int endk = (c == 7 && k == 2) ? Ord<N>::n_tab : (k < 2 ? Ord<N>::off(c, k + 1) : Ord<N>::off(c + 1, 0));
          int cntnz = 0;
          for (int q2 = 0; q2 < nrow * ncol; ++q2) cntnz += pa[q2] != 0.0;
          if (cntnz != endk - off) { err = "advection block sparsity differs from the compiled stencil"; return PN_ERR_INVALID; }
          for (int kk = off; kk < endk; ++kk) {
            const double v = pa[(long long)Ord<N>::rc[kk][0] * ncol + Ord<N>::rc[kk][1]];
            if (std::fabs(v - Ord<N>::val[kk]) > 1e-14 * std::fabs(Ord<N>::val[kk])) {
              err = "the batched path compiles the closed-form coupling blocks; the descriptor's blocks differ";
              return PN_ERR_INVALID;
            }
          }
          pa += (long long)nrow * ncol;
        }
      checked_advection.assign(d->advection, d->advection + L.n_adv);
    }
    double *bf, *ba, *bm;
    T *btf, *bta;
    if ((rc = stage(bf, cpd(d->boundary_fwd, L.n_bnd)))) return rc;
    if ((rc = stage(ba, cpd(d->boundary_adj, L.n_bnd)))) return rc;
    if ((rc = stage(btf, conv(d->boundary_fwd, L.n_bnd)))) return rc;
    if ((rc = stage(bta, conv(d->boundary_adj, L.n_bnd)))) return rc;
    std::vector<double> beam = cpd(d->beam_face, L.n_beam);
    // FP32: scale the beam source so the state stays near unity (a power of two: exact)
    I.scale_g = 1.0;
    if (sizeof(T) == 4) {
      double gmax = 0.0, bmax = 0.0;
      for (double v : beam) gmax = std::max(gmax, std::fabs(v));
      for (int q2 = 0; q2 < ns; ++q2) bmax = std::max(bmax, std::fabs(d->fwd_bc[q2]));
      for (int q2 = 0; q2 <= ns; ++q2) bmax = std::max(bmax, std::fabs(d->adj_int_bc[q2]));
      const double m = gmax * bmax;
      if (m > 0.0 && std::isfinite(m)) I.scale_g = std::ldexp(1.0, -(int)std::lround(std::log2(m)));
    }
    if ((rc = stage(bm, beam.empty() ? std::vector<double>(1, 0.0) : beam))) return rc;
    {
      long long o = 0;
      for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 8; ++c)
          if (class_bit(c, k)) {
            I.bmat_f[k][c] = bf + o;
            I.bmat_a[k][c] = ba + o;
            I.bmt_f[k][c] = btf + o;
            I.bmt_a[k][c] = bta + o;
            o += (long long)L.nm[c] * L.nm[class_switch(c, k)];
          }
      for (int c = 4; c < 8; ++c) I.beam[c] = bm + L.beam_off[c];
    }
    if ((rc = alloc(I.acs, L.n_eee_cells * nr))) return rc;
    if ((rc = alloc(I.noa, L.n_eee_cells * ne))) return rc;
    if ((rc = alloc(I.wint, L.n_eee_cells * nr))) return rc;
    if ((rc = alloc(I.wsum, L.n_eee_cells * nr))) return rc;
    if ((rc = alloc(I.wsrc, L.n_eee_cells * nr))) return rc;
    if ((rc = alloc(I.ibar, nr))) return rc;
    if ((rc = alloc(I.out_mul, 1))) return rc;
    if ((rc = alloc(I.I, nr))) return rc;
    if ((rc = alloc(I.integral, (long long)(ns + 1) * nr))) return rc;
    // work segments
    std::vector<int> faces;
    struct Tmp { int cls; int lo[3], ext[3]; int f0, nf; };
    std::vector<Tmp> per;
    for (int c = 0; c < 8; ++c) {
      if (!L.active[c]) continue;
      Tmp t{};
      t.cls = c;
      int ilo[3], ihi[3];
      for (int k = 0; k < 3; ++k) {
        const int nn = L.shape[c][k];
        if (!L.act[k]) { ilo[k] = 0; ihi[k] = 1; t.lo[k] = 0; t.ext[k] = 1; }
        else if (class_bit(c, k)) { ilo[k] = 1; ihi[k] = nn - 1; t.lo[k] = 1; t.ext[k] = std::max(0, nn - 2); }
        else { ilo[k] = 0; ihi[k] = nn; t.lo[k] = 1; t.ext[k] = std::max(0, nn - 2); }
      }
      t.f0 = (int)faces.size();
      // cells on a face of an axis along which the class is even, in row-major order: whole
      // rows on a z or y face plane, only the x end points elsewhere (O(surface), not O(volume))
      auto on_face = [&](int k, int v) {
        return L.act[k] && !class_bit(c, k) && (v == 0 || v == L.shape[c][k] - 1);
      };
      for (int kz = ilo[2]; kz < ihi[2]; ++kz)
        for (int jy = ilo[1]; jy < ihi[1]; ++jy) {
          if (on_face(2, kz) || on_face(1, jy)) {
            for (int ix = ilo[0]; ix < ihi[0]; ++ix) faces.push_back(pack_cell(ix, jy, kz));
          } else if (L.act[0] && !class_bit(c, 0)) {
            const int last = L.shape[c][0] - 1;
            if (ilo[0] <= 0 && 0 < ihi[0]) faces.push_back(pack_cell(0, jy, kz));
            if (last > 0 && ilo[0] <= last && last < ihi[0]) faces.push_back(pack_cell(last, jy, kz));
          }
        }
      t.nf = (int)faces.size() - t.f0;
      per.push_back(t);
    }
    int* fd;
    if ((rc = stage(fd, faces.empty() ? std::vector<int>(1, 0) : faces))) return rc;
    int nblk[3] = {0, 0, 0};
    for (const Tmp& t : per) {
      for (int list = 0; list < 3; ++list) {
        if (list < 2 && class_parity(t.cls) != list) continue;
        if (t.ext[0] > 0 && t.ext[1] > 0 && t.ext[2] > 0) {
          Seg& g = I.seg[list][I.nseg[list]++];
          g.cls = t.cls;
          g.kind = 0;
          g.block0 = nblk[list];
          for (int k = 0; k < 3; ++k) { g.lo[k] = t.lo[k]; g.ext[k] = t.ext[k]; }
          g.tile_x = (t.ext[1] > 1 || t.ext[2] > 1) ? 32 : BLOCK;
          g.tiles_x = (t.ext[0] + g.tile_x - 1) / g.tile_x;
          g.tiles_y = (t.ext[1] + BLOCK / g.tile_x - 1) / (BLOCK / g.tile_x);
          g.nblocks = g.tiles_x * g.tiles_y * t.ext[2];
          nblk[list] += g.nblocks;
        }
        if (t.nf > 0) {
          Seg& g = I.seg[list][I.nseg[list]++];
          g.cls = t.cls;
          g.kind = 1;
          g.block0 = nblk[list];
          g.tile_x = BLOCK;
          g.tiles_x = g.tiles_y = 1;
          g.n_face = t.nf;
          g.faces = fd + t.f0;
          g.nblocks = (t.nf + BLOCK - 1) / BLOCK;
          nblk[list] += g.nblocks;
        }
      }
    }
    if (nblk[0] == 0 || nblk[1] == 0) { err = "grid too small: a parity has no cells"; return PN_ERR_INVALID; }
    return PN_OK;
  }

  // --------------------------------------------------------------------------------------------
  int launch(int list, int mode, int j, int sub, double* part, bool adj, bool integ) {
    if constexpr (std::is_same<T, float>::value && (DIMS == 3 || DIMS == 7)) {
      if (use_tma) return integ ? launch_tma_int(j) : launch_tma(list, mode, j, sub, part, adj);
    }
    const int x = integ ? j - 1 : j;   // integrate at iteration j includes the solves with ns == j
    const int nt = tiles_active(integ ? 2 : list, x);
    if (nt == 0) return PN_OK;
    BLaunch<T> a;
    a.inst = dinst;
    a.tiles = dtiles[integ ? 2 : list];
    a.list = integ ? 2 : list;
    a.mode = mode;
    a.j = j;
    a.sub = sub;
    a.K = K;
    a.partial = part;
    a.pr = pr;
    a.n_tiles = nt;
    a.tpb = tiles_per_block(nt);
    const int grid = (nt + a.tpb - 1) / a.tpb;
    if (integ)
      batch_integrate_kernel<T, N, DIMS><<<grid, BLOCK, 0, ls>>>(a);
    else if (adj)
      batch_substep_kernel<T, N, true, DIMS><<<grid, BLOCK, 0, ls>>>(a);
    else
      batch_substep_kernel<T, N, false, DIMS><<<grid, BLOCK, 0, ls>>>(a);
    PN_CUDA(cudaGetLastError());
    ++nl;
    return PN_OK;
  }

  // TMA path of a sub-step: every target cell (face tiles compute their ghosts in place)
  int launch_tma(int list, int mode, int j, int sub, double* part, bool adj) {
    if constexpr (std::is_same<T, float>::value && (DIMS == 3 || DIMS == 7)) {
      // solves active at step j (a fused launch also runs step j - 1)
      const int jmin = sub == 4 ? j - 1 : j;
      int last = -1;
      for (int q = 0; q < n; ++q)
        if (hinst[q].ns > jmin) last = q;
      if (last < 0) return PN_OK;
      const int nb = tend[list][last];
      if (nb > 0) {
        TLaunch<N> a;
        a.inst = dinst;
        a.solves = dsolves;
        a.tiles = dttl[list];
        a.maps = dmaps;
        a.rows = static_cast<const ArgRow<N>*>(drows);
        a.partial = part;
        a.status = dstatus;
        a.test_expire = test_expire ? dstatus + 1 : nullptr;
        a.pr = pr;
        a.n_tiles = nb;
        a.mode = mode;
        a.j = j;
        a.sub = sub;
        a.K = K;
        if (sweep) {
          rec_steps.push_back(TStep{adj ? (int)TS_ADJ : (int)TS_FWD, list, mode, j, sub, nb, 0, 0, part});
          return PN_OK;
        }
        const int grid = std::min(nb, tma_grid[adj ? 1 : 0]);
        if (par) {
          if constexpr (kPar) {
            if (adj)
              batch_par_kernel<N, true><<<grid, TB, par_stage, ls>>>(a);
            else
              batch_par_kernel<N, false><<<grid, TB, par_stage, ls>>>(a);
          }
        } else {
          if (adj)
            batch_tma_kernel<N, true, DIMS><<<grid, NTS, TmaLayout<N, DIMS>::SMEM, ls>>>(a);
          else
            batch_tma_kernel<N, false, DIMS><<<grid, NTS, TmaLayout<N, DIMS>::SMEM, ls>>>(a);
        }
        PN_CUDA(cudaGetLastError());
        ++nl;
      }
    } else {
      (void)list; (void)mode; (void)j; (void)sub; (void)part; (void)adj;
    }
    return PN_OK;
  }

  // TMA path of the density integral at iteration j: every cell of every class
  int launch_tma_int(int j) {
    if constexpr (std::is_same<T, float>::value && (DIMS == 3 || DIMS == 7)) {
      int last = -1;
      for (int q = 0; q < n; ++q)
        if (hinst[q].ns >= j) last = q;   // the integral at iteration j includes solves with ns == j
      if (last < 0) return PN_OK;
      const int nb = tend[2][last];
      if (nb > 0) {
        TILaunch<N> a;
        a.inst = dinst;
        a.solves = dsolves;
        a.tiles = dttl[2];
        a.maps = dmaps;
        a.rows = static_cast<const IntRow<N>*>(dirows);
        a.status = dstatus;
        a.n_tiles = nb;
        a.it = j;
        a.K = K;
        if (sweep) {
          rec_steps.push_back(TStep{(int)TS_INT, 2, BM_ADJOINT, j, 0, nb, 0, 0, nullptr});
          return PN_OK;
        }
        batch_tma_int_kernel<N, DIMS><<<std::min(nb, tma_int_grid), NTS, TmaIntLayout<N, DIMS>::SMEM, ls>>>(a);
        PN_CUDA(cudaGetLastError());
        ++nl;
      }
    } else {
      (void)j;
    }
    return PN_OK;
  }

  // forward steps j = top down to bot (the forward sweep with intensity partials, or a recomputed
  // segment): sub-steps 1, 2, 3 per step, or with TMA tiles sub-step 3 of each step fused with
  // sub-step 1 of the next
  int fwd_steps(int top, int bot, int mode, bool partials) {
    int rc;
    auto part = [&](int j) { return partials ? partial + (long long)(max_ns - j - 1) * n_ptiles * pr : nullptr; };
    if (!use_tma) {
      for (int j = top; j >= bot; --j) {
        if ((rc = launch(1, mode, j, 1, nullptr, false, false))) return rc;
        if ((rc = launch(0, mode, j, 2, part(j), false, false))) return rc;
        if ((rc = launch(1, mode, j, 3, nullptr, false, false))) return rc;
      }
      return PN_OK;
    }
    if ((rc = launch(1, mode, top, 1, nullptr, false, false))) return rc;
    for (int j = top; j >= bot; --j) {
      if ((rc = launch(0, mode, j, 2, part(j), false, false))) return rc;
      if ((rc = launch(1, mode, j, j > bot ? 4 : 3, nullptr, false, false))) return rc;
    }
    return PN_OK;
  }

  // adjoint iteration a: density integral on state a, then the three adjoint sub-steps
  int adj_iter(int a) {
    int rc;
    if ((rc = launch(2, BM_ADJOINT, a, 0, nullptr, false, true))) return rc;
    for (int sub = 1; sub <= 3; ++sub)
      if ((rc = launch(sub == 2 ? 0 : 1, BM_ADJOINT, a, sub, nullptr, true, false))) return rc;
    return PN_OK;
  }

  int record(bool fwd) {
    int rc;
    dim3 gz(64, n);
    if (fwd) {
      if (!planning) {
        batch_zero_kernel<T><<<gz, 256, 0, ls>>>(dinst, 0);
        PN_CUDA(cudaGetLastError());
      }
      if ((rc = fwd_steps(max_ns - 1, 0, BM_FORWARD, true))) return rc;
      if ((rc = flush_sweep(true))) return rc;
      if (!planning) {
        batch_reduce_kernel<T><<<dim3(max_ns, n), 128, 0, ls>>>(dinst, partial, max_ns, n_ptiles, pr);
        batch_final_kernel<T><<<n, 32, 0, ls>>>(dinst);
        PN_CUDA(cudaGetLastError());
      }
      nl += 3;
    } else {
      if (!planning) {
        batch_zero_kernel<T><<<gz, 256, 0, ls>>>(dinst, 1);
        PN_CUDA(cudaGetLastError());
      }
      nl += 1;
      // iterations on the kept head, then segments [s0, s0 + K) after recomputing s0 + 1 .. s0 + K - 1;
      // iteration max_ns is the final accumulation of the longest solves on the zero state
      for (int a = 0; a < std::min(A, max_ns + 1); ++a)
        if ((rc = adj_iter(a))) return rc;
      for (int s0 = A; s0 <= max_ns; s0 += K) {
        const int top = std::min(s0 + K, max_ns) - 1;
        if (top >= s0 + 1 && (rc = fwd_steps(top, s0 + 1, BM_RECOMPUTE, false))) return rc;
        for (int a = s0; a < std::min(s0 + K, max_ns + 1); ++a)
          if ((rc = adj_iter(a))) return rc;
      }
      if ((rc = flush_sweep(false))) return rc;
    }
    return PN_OK;
  }

  // The recorded TMA steps of a sweep: while planning, turned into the sweep's plan (item offsets,
  // and per step and solve the step it waits for and its tile count); while capturing, one
  // cooperative launch of batch_sweep_kernel over the planned steps.
  int flush_sweep(bool fwd) {
    if constexpr (std::is_same<T, float>::value && (DIMS == 3 || DIMS == 7)) {
      if (!sweep || rec_steps.empty()) return PN_OK;
      SweepPlan& P = plans[fwd ? 0 : 1];
      if (planning) {
        const int ns = (int)rec_steps.size();
        std::vector<int> dep((size_t)ns * n, -1), need((size_t)ns * n, 0), last(n, -1);
        int items = 0;
        for (int k = 0; k < ns; ++k) {
          TStep& st = rec_steps[k];
          st.first = items;
          items += st.n_tiles;
          int prev = 0;
          for (int q = 0; q < n && prev < st.n_tiles; ++q) {
            const int end = std::min(tend[st.list][q], st.n_tiles);
            const int cnt = end - prev;
            prev = end;
            if (cnt <= 0) continue;
            dep[(size_t)k * n + q] = last[q];
            need[(size_t)k * n + q] = cnt;
            last[q] = k;
          }
        }
        // dep holds step indices; the kernel reads the tile count of the step it waits for
        std::vector<int> need_dep((size_t)ns * n, 0);
        for (int k = 0; k < ns; ++k)
          for (int q = 0; q < n; ++q) {
            const int d = dep[(size_t)k * n + q];
            if (d >= 0) need_dep[(size_t)k * n + q] = need[(size_t)d * n + q];
          }
        int rc;
        if ((rc = upload(P.steps, rec_steps))) return rc;
        if ((rc = upload(P.dep, dep))) return rc;
        if ((rc = upload(P.need, need_dep))) return rc;
        P.n_steps = ns;
        P.n_items = items;
        rec_steps.clear();
        return PN_OK;
      }
      if ((int)rec_steps.size() != P.n_steps) {
        err = "internal: the sweep differs from its plan";
        return PN_ERR_INVALID;
      }
      rec_steps.clear();
      PN_CUDA(cudaMemsetAsync(done_d, 0, sizeof(int) * (size_t)P.n_steps * n, ls));
      TSweep<N> S;
      std::memset(&S, 0, sizeof(S));
      S.inst = dinst;
      S.solves = dsolves;
      for (int l = 0; l < 3; ++l) S.tiles[l] = dttl[l];
      S.maps = dmaps;
      S.rows = static_cast<const ArgRow<N>*>(drows);
      S.irows = static_cast<const IntRow<N>*>(dirows);
      S.status = dstatus;
      S.test_expire = test_expire ? dstatus + 1 : nullptr;
      S.steps = P.steps;
      S.dep = P.dep;
      S.need = P.need;
      S.done = done_d;
      S.n_steps = P.n_steps;
      S.n_items = P.n_items;
      S.n_solves = n;
      S.pr = pr;
      S.K = K;
      S.par = par ? 1 : 0;
      cudaLaunchConfig_t cfg;
      std::memset(&cfg, 0, sizeof(cfg));
      cfg.gridDim = dim3((unsigned)std::min(P.n_items, sweep_grid));
      cfg.blockDim = dim3(NTS);
      cfg.dynamicSmemBytes = sweep_smem();
      cfg.stream = ls;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      PN_CUDA(cudaLaunchKernelEx(&cfg, batch_sweep_kernel<N, DIMS>, S));
      ++nl;
    } else {
      (void)fwd;
    }
    return PN_OK;
  }

  int sweep_smem() const {
    const int sub = par ? par_stage : TmaLayout<N, DIMS>::SMEM;
    return std::max(sub, (int)TmaIntLayout<N, DIMS>::SMEM);
  }

  // plan both sweeps (before the graphs are captured) and size the persistent grid
  int plan_sweeps() {
    if constexpr (std::is_same<T, float>::value && (DIMS == 3 || DIMS == 7)) {
      int rc;
      PN_CUDA(cudaFuncSetAttribute(batch_sweep_kernel<N, DIMS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   sweep_smem()));
      int occ = 0;
      PN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_sweep_kernel<N, DIMS>, NTS, sweep_smem()));
      if (cta_cap > 0) occ = std::min(occ, cta_cap);
      if (occ < 1) {
        sweep = false;
        return PN_OK;
      }
      sweep_grid = occ * sms;
      sweep = true;
      planning = true;
      ls = nullptr;
      rc = record(true);
      if (!rc) rc = record(false);
      planning = false;
      rec_steps.clear();
      nl = 0;
      if (rc) return rc;
      const long long cells = (long long)std::max(plans[0].n_steps, plans[1].n_steps) * n;
      if ((rc = alloc(done_d, std::max(cells, 1LL)))) return rc;
    }
    return PN_OK;
  }

  int capture(cudaGraphExec_t& exec, bool fwd) {
    cudaGraph_t graph = nullptr;
    nl = 0;
    PN_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    ls = cap;
    int rc = record(fwd);
    cudaError_t e = cudaStreamEndCapture(cap, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) {
      err = std::string("stream capture: ") + cudaGetErrorString(e);
      return PN_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      err = std::string("graph instantiate: ") + cudaGetErrorString(e);
      return PN_ERR_CUDA;
    }
    (fwd ? nl_f : nl_a) = nl;
    return PN_OK;
  }

  // The call's solve pointers go to the device in the parameters of a small kernel: parameters
  // are captured at launch, so the call does not wait for the stream (a copy from pageable host
  // memory may wait for it to drain).
  int put_io(const BIo* io_host, cudaStream_t s) {
    IoChunk c;
    for (int q0 = 0; q0 < n; q0 += IoChunk::MAX) {
      c.dst = dio + q0;
      c.n = std::min(IoChunk::MAX, n - q0);
      for (int q = 0; q < c.n; ++q) c.v[q] = io_host[members[q0 + q]];
      batch_put_io_kernel<<<1, 128, 0, s>>>(c);
      PN_CUDA(cudaGetLastError());
    }
    return PN_OK;
  }

  // order `s` after the creation uploads; zero the tapes and densities once
  int prepare(cudaStream_t s) {
    PN_CUDA(cudaStreamWaitEvent(s, ev_up, 0));
    if (!zeroed) {
      for (auto& z : zero_ranges) PN_CUDA(cudaMemsetAsync(z.first, 0, z.second, s));
      zeroed = true;
    }
    return PN_OK;
  }

  int forward(const BIo* io_host, cudaStream_t s) override {
    int rc;
    if ((rc = prepare(s))) return rc;
    // the status word reports the waits of this forward and the adjoint that follows it
    if (dstatus) PN_CUDA(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
    if ((rc = put_io(io_host, s))) return rc;
    batch_load_kernel<T><<<dim3(256, n), 256, 0, s>>>(dinst, dio);
    PN_CUDA(cudaGetLastError());
    if (direct) {
      ls = s;
      nl = 0;
      if ((rc = record(true))) return rc;
      nl_f = nl;
    } else {
      PN_CUDA(cudaGraphLaunch(gf, s));
    }
    batch_copy_I_kernel<T><<<n, 32, 0, s>>>(dinst, dio);
    PN_CUDA(cudaGetLastError());
    return PN_OK;
  }

  int adjoint(const BIo* io_host, cudaStream_t s) override {
    int rc;
    if ((rc = prepare(s))) return rc;
    if ((rc = put_io(io_host, s))) return rc;
    batch_prep_ibar_kernel<T><<<n, 32, 0, s>>>(dinst, dio, sizeof(T) == 4 ? 1 : 0);
    batch_prep_src_kernel<T><<<dim3(64, n), 256, 0, s>>>(dinst);
    PN_CUDA(cudaGetLastError());
    if (direct) {
      ls = s;
      nl = 0;
      if ((rc = record(false))) return rc;
      nl_a = nl;
    } else {
      PN_CUDA(cudaGraphLaunch(ga, s));
    }
    batch_store_kernel<T><<<dim3(256, n), 256, 0, s>>>(dinst, dio);
    PN_CUDA(cudaGetLastError());
    return PN_OK;
  }
};

}  // namespace pn
