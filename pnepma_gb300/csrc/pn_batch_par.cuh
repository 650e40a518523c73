// pn_batch_par.cuh -- FP32 2D sub-steps on parity tiles.
//
// In 2D the four active classes split into two parities, each with two target classes that read
// the same two neighbour classes: parity 0 updates eee and ooe from oee and eoe, parity 1 updates
// eoe and oee from ooe and eee.  A parity tile is one 32 x 4 position of both targets of a parity
// in one CTA: the two target boxes (32 x 4), one box per neighbour class (36 x 5, covering the x
// and y stencils of both targets at once), and both targets' densities.  Against a tile per
// target class (a 40 x 4 x-neighbour box and a 32 x 5 y-neighbour box each) a neighbour value is
// staged once instead of twice, and the shared memory per target point drops by about a third,
// so more points are in flight per SM.  Each thread updates one point of each target, with
// substep_cell's arithmetic (bit-identical states and gradients to the generic kernels).
#pragma once

#include "pn_batch_tma.cuh"

namespace pn {

// resident CTAs per SM the parity-tile kernel is compiled for (shared memory allows four)
#ifndef PN_PAR_MINB
#define PN_PAR_MINB 4
#endif

constexpr int NBW = 36;            // neighbour box width: x0 - 4 .. x0 + 31, or x0 .. x0 + 35
constexpr int NBH = TY + 1;        // neighbour box rows
constexpr int PLN = NBW * NBH;     // floats per moment plane of a neighbour box

// the targets of parity p (A, B) and the neighbour classes F1 = A ^ 4 = B ^ 2, F2 = A ^ 2 = B ^ 4
__host__ __device__ constexpr int par_a(int p) { return p == 0 ? 0 : 2; }
__host__ __device__ constexpr int par_b(int p) { return p == 0 ? 6 : 4; }
// a neighbour box's origin relative to the tile: x0 if the class is odd in x (its readers use
// i .. i + 1 or i), else x0 - 4 (i - 1 .. i, or i); y0 if odd in y, else y0 - 1
__host__ __device__ constexpr int nb_dx(int F) { return ((F >> 2) & 1) ? 0 : -XO; }
__host__ __device__ constexpr int nb_dy(int F) { return ((F >> 1) & 1) ? 0 : -1; }

// target lanes of one class in a parity tile: columns [x lo, x hi), rows [y lo, y hi)
__host__ __device__ inline int par_ext(int xlo, int xhi, int ylo, int yhi) {
  return xlo | (xhi << 8) | (ylo << 16) | (yhi << 24);
}

template <int N>
struct ParLayout {
  static constexpr int maxn(int a, int b) { return a > b ? a : b; }
  static constexpr int al(int b) { return (b + 127) / 128 * 128; }
  static constexpr int NA = maxn(Ord<N>::n(0), Ord<N>::n(2));   // A: eee / eoe
  static constexpr int NB = maxn(Ord<N>::n(6), Ord<N>::n(4));   // B: ooe / oee
  static constexpr int N1 = maxn(Ord<N>::n(4), Ord<N>::n(6));   // F1: oee / ooe
  static constexpr int N2 = maxn(Ord<N>::n(2), Ord<N>::n(0));   // F2: eoe / eee
  static constexpr int OWNA = 0;
  static constexpr int OWNB = OWNA + al(NA * PLO * 4);
  static constexpr int NB1 = OWNB + al(NB * PLO * 4);
  static constexpr int NB2 = NB1 + al(N1 * PLN * 4);
  static constexpr int ARG = NB2 + al(N2 * PLN * 4);   // two rows (a fused launch's steps)
  static constexpr int TIL = ARG + 2 * (int)sizeof(ArgRow<N>);
  static constexpr int SOL = TIL + (int)sizeof(TTile);
  static constexpr int RHOA = al(SOL + (int)sizeof(TSolve));
  // densities of A then B, ne planes each: the stage size depends on the group's elements
  static constexpr int rho_b(int ne) { return RHOA + ne * PLO * 4; }
  static constexpr int smem(int ne) { return RHOA + 2 * ne * PLO * 4; }
};

// Issue a parity tile's loads (one thread); `tt` is the tile record in global memory.  PART 0:
// all of them; 1: all but the target boxes (and the barrier's byte count for all); 2: the target
// boxes only.
template <int N, bool ADJ, int PART = 0>
__device__ __forceinline__ void par_issue(const TLaunch<N>& L, const TTile& tt, unsigned char* st,
                                          unsigned long long* bar) {
  using LY = ParLayout<N>;
  const int p = tt.cls;
  const int A = par_a(p), B = par_b(p), F1 = A ^ 4, F2 = A ^ 2;
  const int nA = class_moments<N>(A), nB = class_moments<N>(B), n1 = class_moments<N>(F1), n2 = class_moments<N>(F2);
  SubSlots sl{0, 0, 0};
  int row, n_rows = 1;
  unsigned arg_dst = 0;
  if (!ADJ) {
    if (L.sub == 4) {
      const int s = slot_index(tt.ns, tt.n_full, tt.n_ck, L.j, L.K, L.mode == BM_RECOMPUTE);
      sl = SubSlots{s, s, s};
      if (fused_first_pass(tt, L.j)) {
        row = tt.arg_fwd + (tt.ns - L.j - 1);
        n_rows = 2;
      } else {
        row = tt.arg_fwd + (tt.ns - L.j);
        arg_dst = (unsigned)sizeof(ArgRow<N>);
      }
    } else {
      sl = sub_slots(tt, L.mode, L.j, L.sub, L.K);
      row = tt.arg_fwd + (tt.ns - L.j - 1);
    }
  } else {
    row = tt.arg_adj + L.j;
  }
  const unsigned bytes = 4u * (unsigned)(PLO * (nA + nB) + PLN * (n1 + n2) + 2 * PLO * tt.ne) +
                         (unsigned)(n_rows * sizeof(ArgRow<N>) + sizeof(TTile) + sizeof(TSolve));
  const CUtensorMap* mp = L.maps + (long long)tt.inst * 8 * TM_KINDS;
  if (PART != 2) mbar_expect_tx(bar, bytes);   // before any of the copies it counts
  if (PART != 1) {
    if (ADJ) {
      if (nA > 0) tma_load_4d(st + LY::OWNA, mp + A * TM_KINDS + TM_LAM_T, tt.x0, tt.y0, tt.z, 0, bar);
      if (nB > 0) tma_load_4d(st + LY::OWNB, mp + B * TM_KINDS + TM_LAM_T, tt.x0, tt.y0, tt.z, 0, bar);
    } else {
      if (nA > 0) tma_load_5d(st + LY::OWNA, mp + A * TM_KINDS + TM_ST_T, tt.x0, tt.y0, tt.z, 0, sl.own, bar);
      if (nB > 0) tma_load_5d(st + LY::OWNB, mp + B * TM_KINDS + TM_ST_T, tt.x0, tt.y0, tt.z, 0, sl.own, bar);
    }
  }
  if (PART == 2) return;
  const int x1 = tt.x0 + nb_dx(F1), y1 = tt.y0 + nb_dy(F1);
  const int x2 = tt.x0 + nb_dx(F2), y2 = tt.y0 + nb_dy(F2);
  if (ADJ) {
    if (n1 > 0) tma_load_4d(st + LY::NB1, mp + F1 * TM_KINDS + TM_LAM_N, x1, y1, tt.z, 0, bar);
    if (n2 > 0) tma_load_4d(st + LY::NB2, mp + F2 * TM_KINDS + TM_LAM_N, x2, y2, tt.z, 0, bar);
  } else {
    if (n1 > 0) tma_load_5d(st + LY::NB1, mp + F1 * TM_KINDS + TM_ST_N, x1, y1, tt.z, 0, sl.from, bar);
    if (n2 > 0) tma_load_5d(st + LY::NB2, mp + F2 * TM_KINDS + TM_ST_N, x2, y2, tt.z, 0, sl.from, bar);
  }
  tma_load_4d(st + LY::RHOA, mp + A * TM_KINDS + TM_RHO, tt.x0, tt.y0, tt.z, 0, bar);
  tma_load_4d(st + LY::rho_b(tt.ne), mp + B * TM_KINDS + TM_RHO, tt.x0, tt.y0, tt.z, 0, bar);
  bulk_load(st + LY::ARG + arg_dst, L.rows + row, (unsigned)(n_rows * sizeof(ArgRow<N>)), bar);
  bulk_load(st + LY::TIL, &tt, (unsigned)sizeof(TTile), bar);
  bulk_load(st + LY::SOL, L.solves + tt.inst, (unsigned)sizeof(TSolve), bar);
}

// The single-axis ghost points target C reads, computed into the shared neighbour boxes
// (ghost_fill's arithmetic, as tile_ghosts).  own: C's target box; fx / fy: the boxes of C ^ 4 and
// C ^ 2.  All threads call this; the caller syncs before reading.
template <int N, int C, int KIND>
__device__ __forceinline__ void par_ghosts(const BInst<float>& I, const TSolve& S, const TTile& tt, int ext,
                                           const float* own, float* fx, float* fy, double bc) {
  constexpr bool ADJ = KIND == 1;
  constexpr int nt = Ord<N>::n(C);
  const int xv0 = ext & 255, xv1 = (ext >> 8) & 255, ylo = (ext >> 16) & 255, yhi = (ext >> 24) & 255;
  if (xv1 <= xv0 || yhi <= ylo) return;
  const double bc_scaled = bc * S.scale_g;
  if constexpr (!((C >> 2) & 1)) {   // even in x: ghosts of F = C ^ 4 at x = 0 and x = n_C
    constexpr int F = C ^ 4;
    constexpr int nf = Ord<N>::n(F);
    if constexpr (nt > 0 && nf > 0) {
      const int ncx = S.n0[C];
      const float* B = ADJ ? I.bmt_a[0][F] : I.bmt_f[0][F];
      constexpr int dy = nb_dy(F);   // F has C's y parity: its row j sits at box row j - y0 - dy
      for (int side = 0; side < 2; ++side) {
        const bool left = side == 0;
        if (left ? (tt.x0 != 0 || xv0 != 0) : tt.x0 + xv1 != ncx) continue;
        const int cc = left ? 0 : ncx - 1 - tt.x0;        // the face cells' column in the target box
        const int gcol = left ? 0 : ncx - tt.x0;          // F's ghost and first interior point (F odd in x:
        const int icol = left ? 1 : ncx - 1 - tt.x0;      // its box starts at x0)
        const bool src = !ADJ && !left;
        const int nrow = yhi - ylo;
        for (int w = threadIdx.x; w < nrow * nf; w += TB) {
          const int ty = ylo + w / nf, r = w % nf;
          float bv = 0.0f;
#pragma unroll
          for (int q = 0; q < nt; ++q) bv = fmaf(B[r * nt + q], own[q * PLO + ty * TX + cc], bv);
          const int j = tt.y0 + ty;
          const float gval =
              src ? float(I.beam[F][((long long)tt.z * S.n1[F] + j) * nf + r] * bc_scaled) : 0.0f;
          const int brow = ty - dy;
          const float interior = fx[r * PLN + brow * NBW + icol];
          fx[r * PLN + brow * NBW + gcol] = left ? 2.0f * (gval - bv) - interior : 2.0f * (bv + gval) - interior;
        }
      }
    }
  }
  if constexpr (!((C >> 1) & 1)) {   // even in y: ghosts of F = C ^ 2 at y = 0 and y = n_C
    constexpr int F = C ^ 2;
    constexpr int nf = Ord<N>::n(F);
    if constexpr (nt > 0 && nf > 0) {
      const int ncy = S.n1[C];
      const float* B = ADJ ? I.bmt_a[1][F] : I.bmt_f[1][F];
      constexpr int dx = nb_dx(F);   // F has C's x parity: its column i sits at box column i - x0 - dx
      const int nx = xv1 - xv0;
      for (int side = 0; side < 2; ++side) {
        const bool left = side == 0;
        if (left ? (tt.y0 != 0 || ylo != 0) : tt.y0 + yhi != ncy) continue;
        const int crow = left ? 0 : ncy - 1 - tt.y0;       // the face cells' row in the target box
        const int grow = left ? 0 : ncy - tt.y0;           // F's ghost and first interior row (F odd in y:
        const int irow = left ? 1 : ncy - 1 - tt.y0;       // its box starts at y0)
        for (int w = threadIdx.x; w < nx * nf; w += TB) {
          const int tx = xv0 + w % nx, r = w / nx;
          float bv = 0.0f;
#pragma unroll
          for (int q = 0; q < nt; ++q) bv = fmaf(B[r * nt + q], own[q * PLO + crow * TX + tx], bv);
          const int bcol = tx - dx;
          const float interior = fy[r * PLN + irow * NBW + bcol];
          fy[r * PLN + grow * NBW + bcol] = left ? 2.0f * (0.0f - bv) - interior : 2.0f * (bv + 0.0f) - interior;
        }
      }
    }
  }
}

// the advection sum of one point of target C from the neighbour boxes: x (box fx), then y (fy)
template <int N, int C, bool NEG>
__device__ __forceinline__ void par_advection(float* acc, const float* fx, const float* fy, int xr, int xl, int yr,
                                              int yl, const TSolve& I) {
  {
    constexpr int F = C ^ 4;
    if constexpr (Ord<N>::n(F) > 0) {
      const float ih = I.inv_h[0];
      auto diff = [&](int q) -> float {
        const float a = fx[q * PLN + xr];
        const float b = fx[q * PLN + xl];
        const float d = NEG ? (b - a) : (a - b);
        return d * ih;
      };
      auto coef = [&](int kk, double lit) -> float {
        (void)kk;
        return float(lit);
      };
      Adv<N, C, 0>::template apply<float>(acc, diff, coef);
    }
  }
  {
    constexpr int F = C ^ 2;
    if constexpr (Ord<N>::n(F) > 0) {
      const float ih = I.inv_h[1];
      auto diff = [&](int q) -> float {
        const float a = fy[q * PLN + yr];
        const float b = fy[q * PLN + yl];
        const float d = NEG ? (b - a) : (a - b);
        return d * ih;
      };
      auto coef = [&](int kk, double lit) -> float {
        (void)kk;
        return float(lit);
      };
      Adv<N, C, 1>::template apply<float>(acc, diff, coef);
    }
  }
}

// One point of target C (tma_update's arithmetic): the new values replace the old ones in C's
// target box.  Intensity partials (eee, forward) accumulate into part.
template <int N, int C, bool ADJ>
__device__ __forceinline__ void par_point(const TLaunch<N>& L, const TTile& tt, int ext, float* own, const float* fx,
                                          const float* fy, const float* rh, const TSolve& I, const ArgRow<N>& ar,
                                          float dt, double* part) {
  constexpr int n = Ord<N>::n(C);
  if constexpr (n > 0) {
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const int xv0 = ext & 255, xv1 = (ext >> 8) & 255, ylo = (ext >> 16) & 255, yhi = (ext >> 24) & 255;
    if (!(tx >= xv0 && tx < xv1 && ty >= ylo && ty < yhi)) return;
    const bool want_part = !ADJ && C == 0 && L.partial != nullptr;
    const int i = tt.x0 + tx, j = tt.y0 + ty;
    const int lo = ty * TX + tx;
    // x neighbours in F = C ^ 4's box (its rows are C's rows): i + 1, i (C even in x) or i, i - 1
    constexpr int Fx = C ^ 4, Fy = C ^ 2;
    const int xrow = (ty - nb_dy(Fx)) * NBW;
    const int xc = tx - nb_dx(Fx);
    const int xr = xrow + (((C >> 2) & 1) ? xc : xc + 1), xl = xr - 1;
    // y neighbours in F = C ^ 2's box (its columns are C's columns): rows j + 1, j or j, j - 1
    const int yc = tx - nb_dx(Fy);
    const int yrow = ty - nb_dy(Fy) + (((C >> 1) & 1) ? 0 : 1);
    const int yr = yrow * NBW + yc, yl = yr - NBW;
    long long ce = 0;
    double wl[MAXR];
    if constexpr (C == 0) {
      ce = ((long long)tt.z * I.n1[0] + j) * I.n0[0] + i;
      const double* wsrc = ADJ ? I.wsrc : I.wint;
#pragma unroll
      for (int r = 0; r < MAXR; ++r) wl[r] = (r < I.nr && (ADJ || want_part)) ? wsrc[ce * I.nr + r] : 0.0;
    }
    float acc[n];
#pragma unroll
    for (int m = 0; m < n; ++m) acc[m] = 0.0f;
    par_advection<N, C, ADJ>(acc, fx, fy, xr, xl, yr, yl, I);
    float rr[MAXE];
    float S = 0.0f;
#pragma unroll
    for (int e = 0; e < MAXE; ++e) {
      rr[e] = e < tt.ne ? rh[e * PLO + lo] : 0.0f;
      S = fmaf(rr[e], ar.s[e], S);
    }
    const float invS = recip(S);
    const float dts = dt * invS;
    constexpr unsigned mask = Ord<N>::deg_mask(C);
    float Cl[N + 1];
    float gl[N + 1];
    cl_sums<float, N, mask>(rr, ar.c, tt.ne, Cl);
#pragma unroll
    for (int l = 0; l <= N; ++l) gl[l] = ((mask >> l) & 1u) ? dts * phi1(-(Cl[l] * dts)) : 0.0f;
    float q0 = 0.0f;
    if constexpr (ADJ && C == 0) {
      double q = 0.0;
#pragma unroll
      for (int r = 0; r < MAXR; ++r)
        if (r < I.nr) q = fma(-ar.sig[r], wl[r], q);
      q0 = float(q);
    }
#pragma unroll
    for (int m = 0; m < n; ++m) {
      const int l = degree_of<N, C>(m);
      const float u = own[m * PLO + lo];
      const float q = (m == 0) ? q0 : 0.0f;
      const float num = fmaf(-Cl[l], u, q - acc[m]);   // (q - A u) - C_l u
      const float unew = fmaf(num, gl[l], u);
      own[m * PLO + lo] = unew;
      if constexpr (C == 0 && !ADJ) {
        if (m == 0 && want_part) {
#pragma unroll
          for (int r = 0; r < MAXR; ++r)
            if (r < I.nr) part[r] += wl[r] * double(unew);
        }
      }
    }
  }
}

// store target class C's box from `box` (thread 0): the adjoint state, or state slot `slot`
template <int N, bool ADJ>
__device__ __forceinline__ void par_store(const TLaunch<N>& L, int inst, int x0, int y0, int z, int C,
                                          const unsigned char* box, int slot) {
  const CUtensorMap* mp = L.maps + ((long long)inst * 8 + C) * TM_KINDS;
  if (ADJ)
    tma_store_4d(mp + TM_LAM_T, x0, y0, z, 0, box);
  else
    tma_store_5d(mp + TM_ST_T, x0, y0, z, 0, slot, box);
}

// One parity tile: one sub-step, or the two of a fused launch, on both targets.  With `next`,
// thread 0 issues that tile's loads other than its target boxes (par_issue part 1) once the last
// pass has finished with the stage, before this tile's stores.
template <int N, int P, bool ADJ>
__device__ __forceinline__ void par_tile_p(const TLaunch<N>& L, const TTile& tt, unsigned char* st,
                                           double (&red)[TB / 32][MAXR], const TTile* next,
                                           unsigned long long* bar) {
  using LY = ParLayout<N>;
  constexpr int A = par_a(P), B = par_b(P), F1 = A ^ 4, F2 = A ^ 2;
  const TSolve& I = *reinterpret_cast<const TSolve*>(st + LY::SOL);
  const ArgRow<N>* rows = reinterpret_cast<const ArgRow<N>*>(st + LY::ARG);
  float* ownA = reinterpret_cast<float*>(st + LY::OWNA);
  float* ownB = reinterpret_cast<float*>(st + LY::OWNB);
  float* nb1 = reinterpret_cast<float*>(st + LY::NB1);
  float* nb2 = reinterpret_cast<float*>(st + LY::NB2);
  const float* rhA = reinterpret_cast<const float*>(st + LY::RHOA);
  const float* rhB = reinterpret_cast<const float*>(st + LY::rho_b(tt.ne));
  const int extA = tt.ext, extB = tt.pad_[0];
  const float half = I.dE * 0.5f;
  const bool fused = !ADJ && L.sub == 4;
  const bool segment = L.mode == BM_RECOMPUTE;
  const int p0 = (fused && !fused_first_pass(tt, L.j)) ? 1 : 0;
  const int p1 = fused ? 2 : 1;
  const BInst<float>& inst = L.inst[tt.inst];
#pragma unroll 1
  for (int pass = p0; pass < p1; ++pass) {
    const bool second = pass == 1;
    const ArgRow<N>& ar = rows[pass];
    const float dt = L.sub == 2 ? I.dE : half;
    // ghosts: A reads F1 along x and F2 along y, B reads F2 along x and F1 along y
    par_ghosts<N, A, ADJ ? 1 : 0>(inst, I, tt, extA, ownA, nb1, nb2, ADJ ? 0.0 : ar.bc);
    par_ghosts<N, B, ADJ ? 1 : 0>(inst, I, tt, extB, ownB, nb2, nb1, ADJ ? 0.0 : ar.bc);
    if (second && threadIdx.x == 0) bulk_wait_read();   // the first pass's stores have read the boxes
    __syncthreads();
    double part[MAXR];
#pragma unroll
    for (int r = 0; r < MAXR; ++r) part[r] = 0.0;
    par_point<N, A, ADJ>(L, tt, extA, ownA, nb1, nb2, rhA, I, ar, dt, part);
    par_point<N, B, ADJ>(L, tt, extB, ownB, nb2, nb1, rhB, I, ar, dt, part);
    if (!ADJ && A == 0 && L.partial != nullptr && tt.pslot >= 0) {   // block-uniform
      const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      if (L.pr <= 1) warp_partials<1>(part, lane, w, L.pr, red);
      else if (L.pr <= 2) warp_partials<2>(part, lane, w, L.pr, red);
      else if (L.pr <= 4) warp_partials<4>(part, lane, w, L.pr, red);
      else warp_partials<8>(part, lane, w, L.pr, red);
      __syncthreads();
      if (threadIdx.x < L.pr) {
        double v = 0.0;
#pragma unroll
        for (int q = 0; q < TB / 32; ++q) v += red[q][threadIdx.x];
        L.partial[(long long)tt.pslot * L.pr + threadIdx.x] = v;
      }
    }
    __syncthreads();   // both target boxes hold the new values
    if (threadIdx.x == 0) {
      int slot = -1;
      if (ADJ) slot = 0;
      else if (!fused) slot = sub_slots(tt, L.mode, L.j, L.sub, L.K).out;
      else if (second || state_kept(tt.ns, tt.n_full, L.j, L.K, segment))
        slot = slot_index(tt.ns, tt.n_full, tt.n_ck, second ? L.j - 1 : L.j, L.K, segment);
      // the tile record is overwritten by the next tile's issue
      const int inst = tt.inst, x0 = tt.x0, y0 = tt.y0, z = tt.z;
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (next != nullptr && pass == p1 - 1) par_issue<N, ADJ, 1>(L, *next, st, bar);
      if (slot >= 0) {
        if (Ord<N>::n(A) > 0) par_store<N, ADJ>(L, inst, x0, y0, z, A, st + LY::OWNA, slot);
        if (Ord<N>::n(B) > 0) par_store<N, ADJ>(L, inst, x0, y0, z, B, st + LY::OWNB, slot);
        bulk_commit();
      }
    }
  }
  (void)F1; (void)F2;
}

template <int N, bool ADJ>
__device__ __forceinline__ void par_tile(const TLaunch<N>& L, const TTile& tt, unsigned char* st,
                                         double (&red)[TB / 32][MAXR], const TTile* next = nullptr,
                                         unsigned long long* bar = nullptr) {
  if (tt.cls == 0) par_tile_p<N, 0, ADJ>(L, tt, st, red, next, bar);
  else par_tile_p<N, 1, ADJ>(L, tt, st, red, next, bar);
}

// Persistent CTAs over a launch's parity tiles (batch_tma_kernel's structure; 2D groups).
template <int N, bool ADJ>
__global__ void __launch_bounds__(TB, PN_PAR_MINB) batch_par_kernel(const __grid_constant__ TLaunch<N> L) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long full[1];
  __shared__ double red[TB / 32][MAXR];
  if ((smem_u32(smem) & 127u) != 0u) {
    if (threadIdx.x == 0) atomicExch(L.status, (int)PN_ERR_INVALID);
    return;
  }
  if (threadIdx.x == 0) {
    mbar_init(&full[0], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int G = gridDim.x;
  unsigned phase = 0;
  for (int k = 0; (int)blockIdx.x + k * G < L.n_tiles; ++k) {
    const int t = blockIdx.x + k * G;
    if (threadIdx.x == 0) {
      if (k == 0) {
        par_issue<N, ADJ, 0>(L, L.tiles[t], smem, &full[0]);
      } else {   // the rest of the tile's loads went out before the previous tile's stores
        bulk_wait_read();   // those stores have read the target boxes
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        par_issue<N, ADJ, 2>(L, L.tiles[t], smem, &full[0]);
      }
    }
    bool ok = mbar_wait_bounded(&full[0], phase);
    if (L.test_expire != nullptr && k == 0 && threadIdx.x == 0 && ok && *(volatile int*)L.test_expire > 0 &&
        atomicSub(L.test_expire, 1) > 0)
      ok = false;   // test hook: report a completed wait as run out (see batch_tma_kernel)
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(L.status, (int)PN_ERR_TIMEOUT);
        mbar_wait_bounded(&full[0], phase);   // let the copies in flight land
        bulk_wait_all();
      }
      __syncthreads();
      return;
    }
    phase ^= 1u;
    const TTile& tt = *reinterpret_cast<const TTile*>(smem + ParLayout<N>::TIL);
    const TTile* next = t + G < L.n_tiles ? L.tiles + t + G : nullptr;
    par_tile<N, ADJ>(L, tt, smem, red, next, &full[0]);
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

}  // namespace pn
