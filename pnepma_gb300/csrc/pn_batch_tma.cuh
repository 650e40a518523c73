// pn_batch_tma.cuh -- FP32 2D/3D sub-steps and density integral of the batched engine with TMA tiles.
//
// The same arithmetic as batch_substep_kernel / batch_integrate_kernel (compiled coupling blocks,
// x, then y, then z), so states and gradients are bit-identical; only the way operands move differs:
//
//   * persistent CTAs walk the tiles of a launch in grid-stride order, so the CTAs resident at
//     any time work on neighbouring tiles;
//   * a tile is 32 x 4 points of one plane of one target class, starting at x0 = 32 bx: lanes
//     outside the class's target cells (its ghost points, or points past the grid) keep the
//     values they were loaded with;
//   * one thread issues, on one mbarrier, cp.async.bulk.tensor loads of the target class's
//     moments (32 x 4 box), the x-neighbour class with its one-point halo (40 x 4 from x0 - 4, the
//     first tile's negative start reading zeros), the y-neighbour class with the halo row the
//     stencil reads (32 x 5 at x0), in 3D the z-neighbour class's planes either side of the
//     tile's plane (32 x 4 x 2), the densities,
//     plus cp.async.bulk copies of the step's coefficient row, the tile record and the solve's
//     arguments; every operand then sits at a compile-time shared-memory offset;
//   * results overwrite the target box in shared memory and go back with one cp.async.bulk.tensor
//     store (bounded by the tensor, aligned at x0).  Stored non-target lanes are ghost points of
//     the target class, which no kernel of a batched solve reads from memory (a face tile computes
//     the ghosts its cells read, below), and no other tile owns them;
//   * a face tile computes the single-axis ghost points its cells read into its staged halo boxes
//     (ghost_fill's arithmetic).
//
// Waits on the mbarrier are bounded (1 s by %globaltimer).  A CTA whose wait runs out records
// PN_ERR_TIMEOUT in the launch's status word, waits (again bounded) for its copies in flight and
// returns.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

namespace pn {

constexpr int TX = 32;              // tile width (points)
// tile height (rows); one thread per point, TB threads per CTA
#ifndef PN_TMA_TY
#define PN_TMA_TY 4
#endif
constexpr int TY = PN_TMA_TY;
constexpr int TB = TX * TY;
// points per thread of the sub-step and density-integral tiles: 1, or 2 x-neighbouring points
// with two-lane FP32 instructions (pn_f32x2.cuh; 36 % fewer instructions, but half the warps per
// SM within the same shared memory, which measured slower on the 2D P11 workload); NTS threads
// per tile
#ifndef PN_TMA_PPT
#define PN_TMA_PPT 1
#endif
constexpr int PPT = PN_TMA_PPT;
constexpr int NTS = TB / PPT;
using LN = Lanes<PPT>;
using LV = LN::V;
constexpr int BW = TX + 8;          // neighbour box width: x0 - 4 .. x0 + 35 (a multiple of 4 floats)
constexpr int XO = 4;               // the tile's first point in a neighbour box
constexpr int PLO = TX * TY;        // floats per moment plane of a target / density box
constexpr int PL4 = BW * TY;        // ... of a 4-row neighbour box
constexpr int PL5 = TX * (TY + 1);  // ... of a 5-row y-neighbour box (32 wide at x0; the y halo row on
                                    // the side the stencil reads)

// minimum resident CTAs per SM the sub-step kernel is compiled for: 5 keeps the adjoint
// instances within 96 registers, so that shared memory, not registers, bounds their occupancy
#ifndef PN_TMA_MINB
#define PN_TMA_MINB 5
#endif

// stages of the tile ring per CTA (1: no prefetch within a CTA, more CTAs per SM)
#ifndef PN_TMA_STAGES
#define PN_TMA_STAGES 1
#endif
constexpr int TSTAGES = PN_TMA_STAGES;

// Coefficients of one step, copied to shared memory with the tile (16-byte multiple).
template <int N>
struct ArgRow {
  float s[MAXE];
  float c[MAXE][N + 1];
  double bc;
  double sig[MAXR];
  double pad_;   // the floats fill 16 (N + 2) bytes; bc, sig and this pad 80
};
static_assert(MAXE == 4 && MAXR == 8, "ArgRow padding assumes 4 elements and 8 lines");

// Coefficients of one adjoint iteration's density integral (fill_int's fields; 16-byte multiple).
template <int N>
struct IntRow {
  float s[MAXE];
  float c[MAXE][N + 1];
  double coef[MAXR];
  double wfac;
  double bc;
};

// One tile of a target class (64 bytes): points x0 .. x0 + 31 (x0 = 32 bx), rows y0 .. y0 + TY - 1,
// plane z; target lanes xv0 <= tx < xv1, rows ty < ey.
struct TTile {
  int inst;     // solve (group order)
  int cls;      // target class
  int x0, y0;
  int ext;      // xv0 | xv1 << 8 | ey << 16
  int pslot;    // partial slot of an eee tile, else -1
  int ns;
  int n_ck;
  int ne;
  int arg_fwd;  // index of the solve's first forward ArgRow
  int arg_adj;  // ... adjoint ArgRow
  int arg_int;  // ... IntRow (n_steps + 1 rows)
  int z;        // plane (0 in 2D)
  int n_full;   // states 0 .. n_full - 1 are all kept (tape head)
  int pad_[2];
};

// The fields of a solve the cell code reads, copied to shared memory with every tile so that no
// per-tile argument costs a dependent global load (16-byte multiple).
struct TSolve {
  float* slots;
  float* lam;
  long long slot_elems;
  double* wint;
  const double* wsrc;
  double* wsum;
  double* rbar[8];
  long long dev_off[8];
  long long ms[8];
  int px[8];
  int n0[8];
  int n1[8];
  int n2[8];
  int xel[MAXR];
  float inv_h[3];
  float dE;
  int nr;
  int ne;
  double scale_g;
};
static_assert(sizeof(TSolve) % 16 == 0, "TSolve must be a 16-byte multiple");
static_assert(sizeof(TTile) % 16 == 0, "TTile must be a 16-byte multiple");

constexpr int PLZ = 2 * PLO;        // floats per moment plane of a z-neighbour box (two planes)

// tensor maps per (solve, class): state (x, y, z, moment, slot) and adjoint state (x, y, z, moment)
// as target boxes and as x / y / z neighbour boxes; densities; rho_bar (FP64)
enum {
  TM_ST_T = 0, TM_ST_X = 1, TM_ST_Y = 2, TM_ST_Z = 3,
  TM_LAM_T = 4, TM_LAM_X = 5, TM_LAM_Y = 6, TM_LAM_Z = 7,
  TM_RHO = 8, TM_RBAR = 9,
  TM_ST_N = 10, TM_LAM_N = 11,   // 36 x 5 neighbour boxes of the 2D parity tiles (pn_batch_par.cuh)
  TM_KINDS = 12
};

template <int N>
struct TLaunch {
  const BInst<float>* inst;
  const TSolve* solves;
  const TTile* tiles;
  const CUtensorMap* maps;      // [solve][8][TM_KINDS]
  const ArgRow<N>* rows;
  double* partial;
  int* status;
  int* test_expire;   // PN_BATCH_TEST_EXPIRE_WAIT: expiries left to report, else NULL
  int pr;
  int n_tiles;
  int mode, j, K;
  int sub;   // 1, 2, 3: that sub-step of energy step j; 4: sub-step 3 of step j, then sub-step 1 of j - 1
};

// the classes a launch updates: z-even ones in 2D (DIMS = 3), all in 3D (DIMS = 7)
template <int N, int DIMS>
struct TmaClasses {
  static constexpr int maxn(int a, int b) { return a > b ? a : b; }
  static constexpr int n_even_z = maxn(maxn(Ord<N>::n(0), Ord<N>::n(2)), maxn(Ord<N>::n(4), Ord<N>::n(6)));
  static constexpr int n_odd_z = maxn(maxn(Ord<N>::n(1), Ord<N>::n(3)), maxn(Ord<N>::n(5), Ord<N>::n(7)));
  static constexpr int NO = DIMS == 7 ? maxn(n_even_z, n_odd_z) : n_even_z;
};

template <int N, int DIMS>
struct TmaLayout {
  static constexpr int NO = TmaClasses<N, DIMS>::NO;
  static constexpr int al(int b) { return (b + 127) / 128 * 128; }
  static constexpr int OWN = 0;
  static constexpr int XN = OWN + al(NO * PLO * 4);
  static constexpr int YN = XN + al(NO * PL4 * 4);
  static constexpr int ZN = YN + al(NO * PL5 * 4);
  static constexpr int RHO = ZN + (DIMS == 7 ? al(NO * PLZ * 4) : 0);
  static constexpr int ARG = RHO + al(MAXE * PLO * 4);      // two rows: steps j and j - 1 of a fused launch
  static constexpr int TIL = ARG + 2 * (int)sizeof(ArgRow<N>);
  static constexpr int SOL = TIL + (int)sizeof(TTile);
  static constexpr int STAGE = al(SOL + (int)sizeof(TSolve));
  static constexpr int SMEM = TSTAGES * STAGE;
};

// Resident CTAs per SM the sub-step and density-integral tile kernels of an order are compiled for,
// i.e. their register cap (65536 / (128 x CTAs)): as many as a tile stage's shared memory allows,
// at most 8 (64 registers), at least PN_TMA_MINB.  The P11 2D stage (40.8 KB) allows 5; small
// orders stage little (P5 3D: 20 KB) and were held to 5-6 CTAs per SM by their registers alone.
template <int N, int DIMS>
struct TmaMinBlocks {
  static constexpr int by_smem = (228 * 1024) / (TmaLayout<N, DIMS>::SMEM + 1024);
  static constexpr int value = by_smem > 8 ? 8 : (by_smem < PN_TMA_MINB ? PN_TMA_MINB : by_smem);
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// wait for phase `parity` of the barrier, at most ~1 s
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* b, unsigned parity) {
  if (mbar_try_wait(b, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(b, parity)) return true;
    if (global_ns() - t0 > 1000000000ull) return false;
  }
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
      : "memory");
}

// shared -> global tensor stores (coordinates >= 0 only), tracked by the bulk async-group
__device__ __forceinline__ void tma_store_4d(const CUtensorMap* map, int c0, int c1, int c2, int c3, const void* src) {
  asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%1, %2, %3, %4}], [%5];"
               ::"l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(src))
               : "memory");
}

__device__ __forceinline__ void tma_store_5d(const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                             const void* src) {
  asm volatile("cp.async.bulk.tensor.5d.global.shared::cta.bulk_group [%0, {%1, %2, %3, %4, %5}], [%6];"
               ::"l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(src))
               : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the stores' shared-memory reads are done (the stage may be overwritten)
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// the stores are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// slot of state j (the index form of bslot)
__device__ __forceinline__ int slot_index(int ns, int n_full, int n_ck, int j, int K, bool segment) {
  if (j >= ns) return 0;
  if (j < n_full) return 1 + j;
  const int r = j - n_full;
  if (r % K == 0) return 1 + n_full + r / K;
  const int w = segment ? (r % K - 1) : (j & 1);
  return 1 + n_full + n_ck + w;
}

// whether state j stays in memory after the forward launches that produce it: kept states (tape
// head, checkpoints) and every state of a recomputed segment; the forward sweep's other states
// are only read by the next step
__device__ __forceinline__ bool state_kept(int ns, int n_full, int j, int K, bool segment) {
  if (segment || j >= ns || j < n_full) return true;
  return (j - n_full) % K == 0;
}

template <int N>
__device__ __forceinline__ int class_moments(int c) {
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

// slots a sub-step reads its own values from, reads its neighbours from, and writes
struct SubSlots {
  int own, from, out;
};

__device__ __forceinline__ SubSlots sub_slots(const TTile& tt, int mode, int j, int sub, int K) {
  const bool segment = mode == BM_RECOMPUTE;
  const int src = slot_index(tt.ns, tt.n_full, tt.n_ck, j + 1, K, segment);
  const int dst = slot_index(tt.ns, tt.n_full, tt.n_ck, j, K, segment);
  return SubSlots{(sub == 3) ? dst : src, (sub == 1) ? src : dst, dst};
}

// A fused launch (sub 4) runs sub-step 3 of step j (pass 0, solves with ns > j) and sub-step 1 of
// step j - 1 (pass 1).  Both update the odd classes from the same even-class values (state j after
// sub-step 2 of step j), so one load serves both: own and neighbour boxes come from state j's slot.
__device__ __forceinline__ bool fused_first_pass(const TTile& tt, int j) { return j < tt.ns; }

// Issue the loads of a tile into stage `st` (one thread).  `tt` must be the tile record in
// global memory (it is also bulk-copied into the stage).
template <int N, bool ADJ, int DIMS>
__device__ __forceinline__ void tma_issue(const TLaunch<N>& L, const TTile& tt, unsigned char* st,
                                          unsigned long long* bar) {
  using LY = TmaLayout<N, DIMS>;
  const int c = tt.cls, cx = c ^ 4, cy = c ^ 2, cz = c ^ 1;
  const int n_own = class_moments<N>(c), n_x = class_moments<N>(cx), n_y = class_moments<N>(cy);
  const int n_z = DIMS == 7 ? class_moments<N>(cz) : 0;
  SubSlots sl{0, 0, 0};
  int row, n_rows = 1;
  unsigned arg_dst = 0;   // byte offset of the first copied row in the stage's two-row area
  if (!ADJ) {
    if (L.sub == 4) {
      // pass 0 reads row (ns - j - 1), pass 1 the next one; a solve that starts at step j - 1
      // has only pass 1
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
  const unsigned bytes = 4u * (unsigned)(PLO * n_own + PL4 * n_x + PL5 * n_y + PLZ * n_z + PLO * tt.ne) +
                         (unsigned)(n_rows * sizeof(ArgRow<N>) + sizeof(TTile) + sizeof(TSolve));
  // the y (z) box starts one row (plane) below the tile for a target odd in y (z): it reads j - 1
  // and j; at the tile for one even in y (z): j and j + 1
  const int ya = tt.y0 - ((c >> 1) & 1);
  const int za = tt.z - (c & 1);
  const int xa = tt.x0 - XO;
  mbar_expect_tx(bar, bytes);
  const CUtensorMap* mp = L.maps + (long long)tt.inst * 8 * TM_KINDS;
  if (ADJ) {
    tma_load_4d(st + LY::OWN, mp + c * TM_KINDS + TM_LAM_T, tt.x0, tt.y0, tt.z, 0, bar);
    if (n_x > 0) tma_load_4d(st + LY::XN, mp + cx * TM_KINDS + TM_LAM_X, xa, tt.y0, tt.z, 0, bar);
    if (n_y > 0) tma_load_4d(st + LY::YN, mp + cy * TM_KINDS + TM_LAM_Y, tt.x0, ya, tt.z, 0, bar);
    if (n_z > 0) tma_load_4d(st + LY::ZN, mp + cz * TM_KINDS + TM_LAM_Z, tt.x0, tt.y0, za, 0, bar);
  } else {
    tma_load_5d(st + LY::OWN, mp + c * TM_KINDS + TM_ST_T, tt.x0, tt.y0, tt.z, 0, sl.own, bar);
    if (n_x > 0) tma_load_5d(st + LY::XN, mp + cx * TM_KINDS + TM_ST_X, xa, tt.y0, tt.z, 0, sl.from, bar);
    if (n_y > 0) tma_load_5d(st + LY::YN, mp + cy * TM_KINDS + TM_ST_Y, tt.x0, ya, tt.z, 0, sl.from, bar);
    if (n_z > 0) tma_load_5d(st + LY::ZN, mp + cz * TM_KINDS + TM_ST_Z, tt.x0, tt.y0, za, 0, sl.from, bar);
  }
  tma_load_4d(st + LY::RHO, mp + c * TM_KINDS + TM_RHO, tt.x0, tt.y0, tt.z, 0, bar);
  bulk_load(st + LY::ARG + arg_dst, L.rows + row, (unsigned)(n_rows * sizeof(ArgRow<N>)), bar);
  bulk_load(st + LY::TIL, &tt, (unsigned)sizeof(TTile), bar);
  bulk_load(st + LY::SOL, L.solves + tt.inst, (unsigned)sizeof(TSolve), bar);
}

// Ghost points of a face tile, computed into its staged neighbour boxes (ghost_fill's arithmetic).
// A class even along an axis reads, at the faces of that axis, a ghost point of the switched class;
// its value depends on the target's values at the face cell (target box) and on the switched
// class's first interior point (neighbour box), both staged.  No other tile reads these ghosts, so
// they are never written to memory.  All threads call this; the caller syncs before reading.
//   own: [n(C)][TY][TX], xb: [n(C^4)][TY][BW] (from x0 - 4), yb: [n(C^2)][TY+1][BW],
//   zb: [n(C^1)][2][TY][TX]
template <int N, int C, int KIND, int DIMS, int NT>
__device__ __forceinline__ void tile_ghosts(const BInst<float>& I, const TSolve& S, const TTile& tt, const float* own,
                                            float* xb, float* yb, float* zb, double bc) {
  constexpr bool ADJ = KIND == 1;
  constexpr int nt = Ord<N>::n(C);
  const int xv0 = tt.ext & 255, xv1 = (tt.ext >> 8) & 255, ey = (tt.ext >> 16) & 255;
  const double bc_scaled = bc * S.scale_g;
  if constexpr (!((C >> 2) & 1)) {   // even in x: ghosts of C ^ 4 at x = 0 and x = n_C
    constexpr int F = C ^ 4;
    constexpr int nf = Ord<N>::n(F);
    if constexpr (nt > 0 && nf > 0) {
      const int ncx = S.n0[C];
      const float* B = ADJ ? I.bmt_a[0][F] : I.bmt_f[0][F];
      for (int side = 0; side < 2; ++side) {
        const bool left = side == 0;
        if (left ? tt.x0 != 0 : tt.x0 + xv1 != ncx) continue;
        // a face tile: the boundary blocks and the beam face come from the full descriptor.
        // Columns: the face cell in the target box; F's ghost (index 0 / n_C) and first interior
        // point (1 / n_C - 1) in the neighbour box, which starts at x0 - 4
        const int cc = left ? 0 : ncx - 1 - tt.x0;
        const int gcol = left ? XO : ncx - tt.x0 + XO;
        const int icol = left ? XO + 1 : ncx - 1 - tt.x0 + XO;
        const bool src = !ADJ && !left;
        for (int w = threadIdx.x; w < ey * nf; w += NT) {
          const int ty = w / nf, r = w % nf;
          float bv = 0.0f;
#pragma unroll
          for (int q = 0; q < nt; ++q) bv = fmaf(B[r * nt + q], own[q * PLO + ty * TX + cc], bv);
          const int j = tt.y0 + ty;
          const float gval =
              src ? float(I.beam[F][((long long)tt.z * S.n1[F] + j) * nf + r] * bc_scaled) : 0.0f;
          const float interior = xb[r * PL4 + ty * BW + icol];
          xb[r * PL4 + ty * BW + gcol] = left ? 2.0f * (gval - bv) - interior : 2.0f * (bv + gval) - interior;
        }
      }
    }
  }
  if constexpr (!((C >> 1) & 1)) {   // even in y: ghosts of C ^ 2 at y = 0 and y = n_C (the y box starts at y0)
    constexpr int F = C ^ 2;
    constexpr int nf = Ord<N>::n(F);
    if constexpr (nt > 0 && nf > 0) {
      const int ncy = S.n1[C];
      const float* B = ADJ ? I.bmt_a[1][F] : I.bmt_f[1][F];
      const int nx = xv1 - xv0;
      for (int side = 0; side < 2; ++side) {
        const bool left = side == 0;
        if (left ? tt.y0 != 0 : tt.y0 + ey != ncy) continue;
        const int crow = left ? 0 : ey - 1;   // the face cells' row in the target box
        const int grow = left ? 0 : ey;       // the ghost row in the y box
        const int irow = left ? 1 : ey - 1;   // the first interior row of F
        for (int w = threadIdx.x; w < nx * nf; w += NT) {
          const int tx = xv0 + w % nx, r = w / nx;
          float bv = 0.0f;
#pragma unroll
          for (int q = 0; q < nt; ++q) bv = fmaf(B[r * nt + q], own[q * PLO + crow * TX + tx], bv);
          const float interior = yb[r * PL5 + irow * TX + tx];
          yb[r * PL5 + grow * TX + tx] = left ? 2.0f * (0.0f - bv) - interior : 2.0f * (bv + 0.0f) - interior;
        }
      }
    }
  }
  if constexpr (DIMS == 7 && !(C & 1)) {   // even in z: ghosts of C ^ 1 at z = 0 and z = n_C (the z box starts at z)
    constexpr int F = C ^ 1;
    constexpr int nf = Ord<N>::n(F);
    if constexpr (nt > 0 && nf > 0) {
      const int ncz = S.n2[C];
      const float* B = ADJ ? I.bmt_a[2][F] : I.bmt_f[2][F];
      const int nx = xv1 - xv0;
      for (int side = 0; side < 2; ++side) {
        const bool left = side == 0;
        if (left ? tt.z != 0 : tt.z != ncz - 1) continue;
        // every target point of the tile is on the face; the ghost plane and F's first interior
        // plane are the two planes of the z box
        const int gpl = left ? 0 : 1, ipl = left ? 1 : 0;
        for (int w = threadIdx.x; w < ey * nx * nf; w += NT) {
          const int r = w / (ey * nx), rest = w % (ey * nx);
          const int ty = rest / nx, tx = xv0 + rest % nx;
          float bv = 0.0f;
#pragma unroll
          for (int q = 0; q < nt; ++q) bv = fmaf(B[r * nt + q], own[q * PLO + ty * TX + tx], bv);
          const float interior = zb[r * PLZ + ipl * PLO + ty * TX + tx];
          zb[r * PLZ + gpl * PLO + ty * TX + tx] = left ? 2.0f * (0.0f - bv) - interior : 2.0f * (bv + 0.0f) - interior;
        }
      }
    }
  }
}

constexpr int ilog2c(int v) { return v <= 1 ? 0 : 1 + ilog2c(v / 2); }

// Sum values v[0 .. V-1] over the lanes of a warp.  Each halving step (lane bits 16, 8, ...) has
// every lane keep half of its values and add its partner's copy of that half, so V values cost
// V - 1 adds; the remaining lane bits then reduce the one value left.  Lane l ends with the sum of
// value (l >> (5 - log2 V)); the first lane of each group writes it to red[w][value].
template <int V, int W>
__device__ __forceinline__ void warp_partials(double* v, int lane, int w, int pr, double (&red)[W][MAXR]) {
  constexpr int levels = ilog2c(V);
  int base = 0;
#pragma unroll
  for (int lv = 0; lv < levels; ++lv) {
    const int h = V >> (lv + 1), o = 16 >> lv;
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < h; ++k) {
      const double give = upper ? v[k] : v[k + h];
      const double keep = upper ? v[k + h] : v[k];
      v[k] = keep + __shfl_xor_sync(0xffffffffu, give, o);
    }
    if (upper) base += h;
  }
#pragma unroll
  for (int o = 16 >> levels; o > 0; o >>= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
  if ((lane & ((32 >> levels) - 1)) == 0 && base < pr) red[w][base] = v[0];
}

// The advection sum of the thread's point(s) from the staged boxes: x, then y, then z
// (advection_sum's order and arithmetic, lane by lane).  With two points per thread the x
// neighbours come from three consecutive values of the neighbour box; y and z neighbours are
// aligned pairs.
template <int N, int C, bool NEG, int DIMS>
__device__ __forceinline__ void staged_advection(LV* acc, const float* xn, const float* yn, const float* zn,
                                                 int xr, int xl, int yr, int yl, int zo, const TSolve& I) {
  {
    constexpr int F = C ^ 4;
    constexpr bool oddx = (C >> 2) & 1;   // then xr is even, else xl is
    if constexpr (Ord<N>::n(F) > 0) {
      const LV ih = LN::splat(I.inv_h[0]);
      auto diff = [&](int q) -> LV {
        LV a, b;
        LN::xpair(xn + q * PL4, xr, xl, oddx, a, b);
        const LV d = NEG ? (b - a) : (a - b);
        return d * ih;
      };
      auto coef = [&](int kk, double lit) -> LV {
        (void)kk;
        return LN::splat(float(lit));
      };
      Adv<N, C, 0>::template apply<LV>(acc, diff, coef);
    }
  }
  {
    constexpr int F = C ^ 2;
    if constexpr (Ord<N>::n(F) > 0) {
      const LV ih = LN::splat(I.inv_h[1]);
      auto diff = [&](int q) -> LV {
        const LV a = LN::ld(yn + q * PL5 + yr);
        const LV b = LN::ld(yn + q * PL5 + yl);
        const LV d = NEG ? (b - a) : (a - b);
        return d * ih;
      };
      auto coef = [&](int kk, double lit) -> LV {
        (void)kk;
        return LN::splat(float(lit));
      };
      Adv<N, C, 1>::template apply<LV>(acc, diff, coef);
    }
  }
  if constexpr (DIMS == 7) {
    constexpr int F = C ^ 1;
    if constexpr (Ord<N>::n(F) > 0) {
      const LV ih = LN::splat(I.inv_h[2]);
      auto diff = [&](int q) -> LV {   // planes: 1 = j (odd) / j + 1 (even), 0 = j - 1 / j
        const LV a = LN::ld(zn + q * PLZ + PLO + zo);
        const LV b = LN::ld(zn + q * PLZ + zo);
        const LV d = NEG ? (b - a) : (a - b);
        return d * ih;
      };
      auto coef = [&](int kk, double lit) -> LV {
        (void)kk;
        return LN::splat(float(lit));
      };
      Adv<N, C, 2>::template apply<LV>(acc, diff, coef);
    }
  }
}

// cl_sums for the thread's lanes (the same sums in the same order per lane)
template <int N, unsigned MASK, int NE>
__device__ __forceinline__ void cl_sums_lanes_n(const LV* rr, const float (*c)[N + 1], LV* Cl) {
#pragma unroll
  for (int l = 0; l <= N; ++l) {
    LV cc = LN::splat(0.0f);
    if ((MASK >> l) & 1u) {
#pragma unroll
      for (int e = 0; e < NE; ++e) cc = fma(rr[e], LN::splat(c[e][l]), cc);
    }
    Cl[l] = cc;
  }
}

template <int N, unsigned MASK>
__device__ __forceinline__ void cl_sums_lanes(const LV* rr, const float (*c)[N + 1], int ne, LV* Cl) {
  switch (ne) {
    case 1: cl_sums_lanes_n<N, MASK, 1>(rr, c, Cl); break;
    case 2: cl_sums_lanes_n<N, MASK, 2>(rr, c, Cl); break;
    case 3: cl_sums_lanes_n<N, MASK, 3>(rr, c, Cl); break;
    default: cl_sums_lanes_n<N, MASK, MAXE>(rr, c, Cl); break;
  }
}

// One update of a staged tile: substep_cell's arithmetic with operands from shared memory; the new
// values replace the old ones in the target box.  `ar` holds the step's coefficients, `dt` its
// (half or full) energy step.  With `settle`, thread 0 waits for the reads of the tile's earlier
// store after the ghosts are formed and before the target box is written.
template <int N, int C, bool ADJ, int DIMS>
__device__ __forceinline__ void tma_update(const TLaunch<N>& L, const TTile& tt, unsigned char* st,
                                           double (&red)[NTS / 32][MAXR], const ArgRow<N>& ar, float dt,
                                           bool settle) {
  using LY = TmaLayout<N, DIMS>;
  constexpr int n = Ord<N>::n(C);
  constexpr bool oddx = (C >> 2) & 1;
  const TSolve& I = *reinterpret_cast<const TSolve*>(st + LY::SOL);
  float* own = reinterpret_cast<float*>(st + LY::OWN);
  tile_ghosts<N, C, ADJ ? 1 : 0, DIMS, NTS>(L.inst[tt.inst], I, tt, own, reinterpret_cast<float*>(st + LY::XN),
                                            reinterpret_cast<float*>(st + LY::YN),
                                            reinterpret_cast<float*>(st + LY::ZN), ADJ ? 0.0 : ar.bc);
  if (settle && threadIdx.x == 0) bulk_wait_read();
  __syncthreads();
  const float* xn = reinterpret_cast<const float*>(st + LY::XN);
  const float* yn = reinterpret_cast<const float*>(st + LY::YN);
  const float* zn = reinterpret_cast<const float*>(st + LY::ZN);
  const float* rh = reinterpret_cast<const float*>(st + LY::RHO);
  // this thread's points: (tx + k, ty), k < PPT
  const int tx = PPT * (threadIdx.x % (TX / PPT)), ty = threadIdx.x / (TX / PPT);
  const int xv0 = tt.ext & 255, xv1 = (tt.ext >> 8) & 255, ey = (tt.ext >> 16) & 255;
  bool vk[PPT];
  bool any = false;
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    vk[k] = tx + k >= xv0 && tx + k < xv1 && ty < ey;
    any = any || vk[k];
  }
  const bool want_part = !ADJ && C == 0 && L.partial != nullptr;
  double part[MAXR];
#pragma unroll
  for (int r = 0; r < MAXR; ++r) part[r] = 0.0;
  if constexpr (n > 0) {
    if (any) {
      const int i = tt.x0 + tx, j = tt.y0 + ty;
      const int lo = ty * TX + tx;                              // the point(s) in the target / density / z boxes
      const int xr = ty * BW + tx + XO + (oddx ? 0 : 1), xl = xr - 1;   // x neighbours: i, i - 1 (odd) or i + 1, i
      const int yr = (ty + 1) * TX + tx, yl = yr - TX;          // rows j, j - 1 (odd) or j + 1, j of the y box
      // the eee cells' per-line weights (intensity or adjoint source), loaded before the stencil
      // so that their latency overlaps it
      long long ce = 0;
      double wl[PPT][MAXR];
      if constexpr (C == 0) {
        ce = ((long long)tt.z * I.n1[0] + j) * I.n0[0] + i;
        const double* wsrc = ADJ ? I.wsrc : I.wint;
        const bool use = ADJ || want_part;
#pragma unroll
        for (int k = 0; k < PPT; ++k)
#pragma unroll
          for (int r = 0; r < MAXR; ++r) wl[k][r] = (r < I.nr && use && vk[k]) ? wsrc[(ce + k) * I.nr + r] : 0.0;
      }
      LV acc[n];
#pragma unroll
      for (int m = 0; m < n; ++m) acc[m] = LN::splat(0.0f);
      staged_advection<N, C, ADJ, DIMS>(acc, xn, yn, zn, xr, xl, yr, yl, lo, I);
      LV rr[MAXE];
      LV S = LN::splat(0.0f);
#pragma unroll
      for (int e = 0; e < MAXE; ++e) {
        rr[e] = e < tt.ne ? LN::ld(rh + e * PLO + lo) : LN::splat(0.0f);
        S = fma(rr[e], LN::splat(ar.s[e]), S);
      }
      const LV invS = LN::rcp(S);
      const LV dts = LN::splat(dt) * invS;
      constexpr unsigned mask = Ord<N>::deg_mask(C);
      LV Cl[N + 1];
      LV gl[N + 1];   // dt phi1_l / S (substep_cell's factors)
      cl_sums_lanes<N, mask>(rr, ar.c, tt.ne, Cl);
#pragma unroll
      for (int l = 0; l <= N; ++l) gl[l] = ((mask >> l) & 1u) ? dts * phi1(LN::neg(Cl[l] * dts)) : LN::splat(0.0f);
      LV q0 = LN::splat(0.0f);
      if constexpr (ADJ && C == 0) {
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          double q = 0.0;
#pragma unroll
          for (int r = 0; r < MAXR; ++r)
            if (r < I.nr) q = fma(-ar.sig[r], wl[k][r], q);
          LN::set(q0, k, float(q));
        }
      }
#pragma unroll
      for (int m = 0; m < n; ++m) {
        const int l = degree_of<N, C>(m);
        const LV u = LN::ld(own + m * PLO + lo);
        const LV q = (m == 0) ? q0 : LN::splat(0.0f);
        const LV num = fma(LN::neg(Cl[l]), u, q - acc[m]);   // (q - A u) - C_l u
        LV unew = fma(num, gl[l], u);
#pragma unroll
        for (int k = 0; k < PPT; ++k)
          if (!vk[k]) LN::set(unew, k, LN::get(u, k));   // lanes outside the target cells keep their values
        LN::st(own + m * PLO + lo, unew);
        if constexpr (C == 0 && !ADJ) {
          if (m == 0 && want_part) {
#pragma unroll
            for (int k = 0; k < PPT; ++k)
#pragma unroll
              for (int r = 0; r < MAXR; ++r)
                if (r < I.nr && vk[k]) part[r] += wl[k][r] * double(LN::get(unew, k));
          }
        }
      }
    }
  }
  if (want_part && tt.pslot >= 0) {   // block-uniform
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // FP64 adds are scarce on this GPU (2 per SM per clock): reduce only the group's lines, V of
    // them at once with V - 1 + log2(32 / V) adds per warp
    if (L.pr <= 1) warp_partials<1>(part, lane, w, L.pr, red);
    else if (L.pr <= 2) warp_partials<2>(part, lane, w, L.pr, red);
    else if (L.pr <= 4) warp_partials<4>(part, lane, w, L.pr, red);
    else warp_partials<8>(part, lane, w, L.pr, red);
    __syncthreads();
    if (threadIdx.x < L.pr) {
      double v = 0.0;
#pragma unroll
      for (int q = 0; q < NTS / 32; ++q) v += red[q][threadIdx.x];
      L.partial[(long long)tt.pslot * L.pr + threadIdx.x] = v;
    }
  }
  __syncthreads();   // the target box holds the new values
}

// store the target box (thread 0): the adjoint state, or state slot `slot`
template <int N, int C, bool ADJ, int DIMS>
__device__ __forceinline__ void tma_store_target(const TLaunch<N>& L, const TTile& tt, unsigned char* st, int slot) {
  using LY = TmaLayout<N, DIMS>;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  const CUtensorMap* mp = L.maps + ((long long)tt.inst * 8 + C) * TM_KINDS;
  if (ADJ)
    tma_store_4d(mp + TM_LAM_T, tt.x0, tt.y0, tt.z, 0, st + LY::OWN);
  else
    tma_store_5d(mp + TM_ST_T, tt.x0, tt.y0, tt.z, 0, slot, st + LY::OWN);
  bulk_commit();
}

template <int N, int C, bool ADJ, int DIMS>
__device__ __forceinline__ void tma_cell(const TLaunch<N>& L, const TTile& tt, unsigned char* st,
                                         double (&red)[NTS / 32][MAXR]) {
  using LY = TmaLayout<N, DIMS>;
  const TSolve& I = *reinterpret_cast<const TSolve*>(st + LY::SOL);
  const ArgRow<N>* rows = reinterpret_cast<const ArgRow<N>*>(st + LY::ARG);
  const float half = I.dE * 0.5f;
  // passes: one sub-step, or the two of a fused launch (the first skipped for a solve that starts
  // at step j - 1); one copy of the update code serves all of them
  const bool fused = !ADJ && L.sub == 4;
  const bool segment = L.mode == BM_RECOMPUTE;
  const int p0 = (fused && !fused_first_pass(tt, L.j)) ? 1 : 0;
  const int p1 = fused ? 2 : 1;
#pragma unroll 1
  for (int pass = p0; pass < p1; ++pass) {
    const bool second = pass == 1;
    // the second update overwrites the target box once the first store has read it
    tma_update<N, C, ADJ, DIMS>(L, tt, st, red, rows[pass], L.sub == 2 ? I.dE : half, second);
    if (threadIdx.x == 0) {
      if (ADJ) {
        tma_store_target<N, C, ADJ, DIMS>(L, tt, st, 0);
      } else if (!fused) {
        tma_store_target<N, C, ADJ, DIMS>(L, tt, st, sub_slots(tt, L.mode, L.j, L.sub, L.K).out);
      } else if (second || state_kept(tt.ns, tt.n_full, L.j, L.K, segment)) {
        const int jj = second ? L.j - 1 : L.j;
        tma_store_target<N, C, ADJ, DIMS>(L, tt, st, slot_index(tt.ns, tt.n_full, tt.n_ck, jj, L.K, segment));
      }
    }
  }
}

template <int N, bool ADJ, int DIMS>
__device__ __forceinline__ void tma_cell_of(const TLaunch<N>& L, const TTile& tt, unsigned char* st,
                                            double (&red)[NTS / 32][MAXR]) {
  if constexpr (DIMS == 7) {
    switch (tt.cls) {
      case 0: tma_cell<N, 0, ADJ, DIMS>(L, tt, st, red); break;
      case 1: tma_cell<N, 1, ADJ, DIMS>(L, tt, st, red); break;
      case 2: tma_cell<N, 2, ADJ, DIMS>(L, tt, st, red); break;
      case 3: tma_cell<N, 3, ADJ, DIMS>(L, tt, st, red); break;
      case 4: tma_cell<N, 4, ADJ, DIMS>(L, tt, st, red); break;
      case 5: tma_cell<N, 5, ADJ, DIMS>(L, tt, st, red); break;
      case 6: tma_cell<N, 6, ADJ, DIMS>(L, tt, st, red); break;
      default: tma_cell<N, 7, ADJ, DIMS>(L, tt, st, red); break;
    }
  } else {
    switch (tt.cls) {
      case 0: tma_cell<N, 0, ADJ, DIMS>(L, tt, st, red); break;
      case 2: tma_cell<N, 2, ADJ, DIMS>(L, tt, st, red); break;
      case 4: tma_cell<N, 4, ADJ, DIMS>(L, tt, st, red); break;
      default: tma_cell<N, 6, ADJ, DIMS>(L, tt, st, red); break;
    }
  }
}

template <int N, bool ADJ, int DIMS>
__global__ void __launch_bounds__(NTS, (TmaMinBlocks<N, DIMS>::value)) batch_tma_kernel(const __grid_constant__ TLaunch<N> L) {
  using LY = TmaLayout<N, DIMS>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long full[TSTAGES];
  __shared__ double red[NTS / 32][MAXR];
  // tensor copies need 128-byte aligned destinations: refuse (uniformly) rather than fault
  if ((smem_u32(smem) & 127u) != 0u) {
    if (threadIdx.x == 0) atomicExch(L.status, (int)PN_ERR_INVALID);
    return;
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < TSTAGES; ++s) mbar_init(&full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int G = gridDim.x;
  const int t0 = blockIdx.x;
  // tiles t0 + k G, k = 0, 1, ...; tile k lives in stage k % TSTAGES, use (k / TSTAGES) of its barrier
  if (threadIdx.x == 0)
    for (int k = 0; k < TSTAGES - 1; ++k) {
      const int t = t0 + k * G;
      if (t < L.n_tiles) tma_issue<N, ADJ, DIMS>(L, L.tiles[t], smem + k * LY::STAGE, &full[k]);
    }
  for (int k = 0; t0 + k * G < L.n_tiles; ++k) {
    const int s = k % TSTAGES;
    const int ka = k + TSTAGES - 1;   // tile issued now, into the stage freed by iteration k - 1
    const int ta = t0 + ka * G;
    if (ta < L.n_tiles && threadIdx.x == 0) {
      bulk_wait_read();   // the stores issued from that stage have read it
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tma_issue<N, ADJ, DIMS>(L, L.tiles[ta], smem + (ka % TSTAGES) * LY::STAGE, &full[ka % TSTAGES]);
    }
    bool ok = mbar_wait_bounded(&full[s], (unsigned)((k / TSTAGES) & 1));
    // test hook: report a wait that has completed (its copies have landed) as run out, once per
    // batch, so that the failure path runs with no copy of this stage in flight
    if (L.test_expire != nullptr && k == 0 && threadIdx.x == 0 && ok && *(volatile int*)L.test_expire > 0 &&
        atomicSub(L.test_expire, 1) > 0)
      ok = false;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(L.status, (int)PN_ERR_TIMEOUT);
        // let the copies still in flight land before the CTA's shared memory is released
        for (int kk = k; kk <= ka; ++kk)
          if (t0 + kk * G < L.n_tiles) mbar_wait_bounded(&full[kk % TSTAGES], (unsigned)((kk / TSTAGES) & 1));
        bulk_wait_all();
      }
      __syncthreads();
      return;
    }
    unsigned char* st = smem + s * LY::STAGE;
    const TTile& tt = *reinterpret_cast<const TTile*>(st + LY::TIL);
    tma_cell_of<N, ADJ, DIMS>(L, tt, st, red);
  }
  if (threadIdx.x == 0) bulk_wait_all();   // every store of this CTA has landed
}

// ---------------------------------------------------------------------------------------------
// density integral of the adjoint (integrate_cell's arithmetic), every class of a solve
// ---------------------------------------------------------------------------------------------
template <int N>
struct TILaunch {
  const BInst<float>* inst;
  const TSolve* solves;
  const TTile* tiles;
  const CUtensorMap* maps;
  const IntRow<N>* rows;
  int* status;
  int n_tiles;
  int it;   // adjoint iteration (tape state it)
  int K;
};

template <int N, int DIMS>
struct TmaIntLayout {
  using B = TmaLayout<N, DIMS>;
  static constexpr int NO = B::NO;
  // the tape state's target box and its neighbours, the densities; the adjoint state and rho_bar
  // are read (and rho_bar written) per point from global memory
  static constexpr int OWN = 0;
  static constexpr int XN = OWN + B::al(NO * PLO * 4);
  static constexpr int YN = XN + B::al(NO * PL4 * 4);
  static constexpr int ZN = YN + B::al(NO * PL5 * 4);
  static constexpr int RHO = ZN + (DIMS == 7 ? B::al(NO * PLZ * 4) : 0);
  static constexpr int ARG = RHO + B::al(MAXE * PLO * 4);
  static constexpr int TIL = ARG + (int)sizeof(IntRow<N>);
  static constexpr int SOL = TIL + (int)sizeof(TTile);
  static constexpr int STAGE = B::al(SOL + (int)sizeof(TSolve));
  static constexpr int SMEM = TSTAGES * STAGE;
};

template <int N, int DIMS>
__device__ __forceinline__ void tma_issue_int(const TILaunch<N>& L, const TTile& tt, unsigned char* st,
                                              unsigned long long* bar) {
  using LY = TmaIntLayout<N, DIMS>;
  const int c = tt.cls, cx = c ^ 4, cy = c ^ 2, cz = c ^ 1;
  const int n_own = class_moments<N>(c), n_x = class_moments<N>(cx), n_y = class_moments<N>(cy);
  const int n_z = DIMS == 7 ? class_moments<N>(cz) : 0;
  const int slot = slot_index(tt.ns, tt.n_full, tt.n_ck, L.it, L.K, true);
  const unsigned bytes = 4u * (unsigned)(PLO * n_own + PL4 * n_x + PL5 * n_y + PLZ * n_z + PLO * tt.ne) +
                         (unsigned)(sizeof(IntRow<N>) + sizeof(TTile) + sizeof(TSolve));
  const int ya = tt.y0 - ((c >> 1) & 1);
  const int za = tt.z - (c & 1);
  const int xa = tt.x0 - XO;
  mbar_expect_tx(bar, bytes);
  const CUtensorMap* mp = L.maps + (long long)tt.inst * 8 * TM_KINDS;
  tma_load_5d(st + LY::OWN, mp + c * TM_KINDS + TM_ST_T, tt.x0, tt.y0, tt.z, 0, slot, bar);
  if (n_x > 0) tma_load_5d(st + LY::XN, mp + cx * TM_KINDS + TM_ST_X, xa, tt.y0, tt.z, 0, slot, bar);
  if (n_y > 0) tma_load_5d(st + LY::YN, mp + cy * TM_KINDS + TM_ST_Y, tt.x0, ya, tt.z, 0, slot, bar);
  if (n_z > 0) tma_load_5d(st + LY::ZN, mp + cz * TM_KINDS + TM_ST_Z, tt.x0, tt.y0, za, 0, slot, bar);
  tma_load_4d(st + LY::RHO, mp + c * TM_KINDS + TM_RHO, tt.x0, tt.y0, tt.z, 0, bar);
  bulk_load(st + LY::ARG, L.rows + tt.arg_int + L.it, (unsigned)sizeof(IntRow<N>), bar);
  bulk_load(st + LY::TIL, &tt, (unsigned)sizeof(TTile), bar);
  bulk_load(st + LY::SOL, L.solves + tt.inst, (unsigned)sizeof(TSolve), bar);
}

template <int N, int C, int DIMS>
__device__ __forceinline__ void tma_int_cell(const TILaunch<N>& L, const TTile& tt, unsigned char* st) {
  using LY = TmaIntLayout<N, DIMS>;
  constexpr int n = Ord<N>::n(C);
  constexpr bool oddx = (C >> 2) & 1;
  const TSolve& I = *reinterpret_cast<const TSolve*>(st + LY::SOL);
  const float* own = reinterpret_cast<const float*>(st + LY::OWN);
  {
    const IntRow<N>& ar0 = *reinterpret_cast<const IntRow<N>*>(st + LY::ARG);
    tile_ghosts<N, C, 2, DIMS, NTS>(L.inst[tt.inst], I, tt, own, reinterpret_cast<float*>(st + LY::XN),
                                    reinterpret_cast<float*>(st + LY::YN), reinterpret_cast<float*>(st + LY::ZN),
                                    ar0.bc);
    __syncthreads();
  }
  if constexpr (n > 0) {
    // this thread's points: (tx + k, ty), k < PPT
    const int tx = PPT * (threadIdx.x % (TX / PPT)), ty = threadIdx.x / (TX / PPT);
    const int xv0 = tt.ext & 255, xv1 = (tt.ext >> 8) & 255, ey = (tt.ext >> 16) & 255;
    bool vk[PPT];
    bool any = false;
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      vk[k] = tx + k >= xv0 && tx + k < xv1 && ty < ey;
      any = any || vk[k];
    }
    if (any) {
      const float* xn = reinterpret_cast<const float*>(st + LY::XN);
      const float* yn = reinterpret_cast<const float*>(st + LY::YN);
      const float* zn = reinterpret_cast<const float*>(st + LY::ZN);
      const float* rh = reinterpret_cast<const float*>(st + LY::RHO);
      const IntRow<N>& ar = *reinterpret_cast<const IntRow<N>*>(st + LY::ARG);
      const int i = tt.x0 + tx, j = tt.y0 + ty;
      const int lo = ty * TX + tx;
      const int xr = ty * BW + tx + XO + (oddx ? 0 : 1), xl = xr - 1;
      const int yr = (ty + 1) * TX + tx, yl = yr - TX;
      // the point(s)' place in the class's device layout (x fastest, pitch px); with two points
      // x is even, so the adjoint state's pairs are 8-byte and rho_bar's 16-byte aligned
      const long long p = ((long long)tt.z * I.n1[C] + j) * I.px[C] + i;
      const long long ms = I.ms[C];
      // the adjoint state, loaded before the stencil so that its latency overlaps it
      const float* la = I.lam + I.dev_off[C] + p;
      LV lam[n];
#pragma unroll
      for (int m = 0; m < n; ++m) lam[m] = LN::ldcg(la + m * ms);   // L2: earlier steps of a sweep launch wrote it
      // the eee cells' line sums
      long long ce = 0;
      double wl[PPT][MAXR];
      if constexpr (C == 0) {
        ce = ((long long)tt.z * I.n1[0] + j) * I.n0[0] + i;
#pragma unroll
        for (int k = 0; k < PPT; ++k)
#pragma unroll
          for (int r = 0; r < MAXR; ++r) wl[k][r] = (r < I.nr && vk[k]) ? __ldcg(&I.wsum[(ce + k) * I.nr + r]) : 0.0;
      }
      LV acc[n];
#pragma unroll
      for (int m = 0; m < n; ++m) acc[m] = LN::splat(0.0f);
      staged_advection<N, C, false, DIMS>(acc, xn, yn, zn, xr, xl, yr, yl, lo, I);
      LV rr[MAXE];
      LV S = LN::splat(0.0f);
#pragma unroll
      for (int e = 0; e < MAXE; ++e) {
        rr[e] = e < tt.ne ? LN::ld(rh + e * PLO + lo) : LN::splat(0.0f);
        S = fma(rr[e], LN::splat(ar.s[e]), S);
      }
      const LV invS = LN::rcp(S);
      constexpr unsigned mask = Ord<N>::deg_mask(C);
      LV Cl[N + 1];
      cl_sums_lanes<N, mask>(rr, ar.c, tt.ne, Cl);
      LV P = LN::splat(0.0f);
      LV R[N + 1];
#pragma unroll
      for (int l = 0; l <= N; ++l) R[l] = LN::splat(0.0f);
#pragma unroll
      for (int m = 0; m < n; ++m) {
        const int l = degree_of<N, C>(m);
        const LV u = LN::ld(own + m * PLO + lo);
        P = fma(lam[m], fma(LN::neg(Cl[l]), u, LN::neg(acc[m])), P);   // 1/S applied once, below (integrate_cell's order)
        R[l] = fma(lam[m], u, R[l]);
      }
      P = P * invS;
      double* rb = I.rbar[C] + p;
#pragma unroll
      for (int e = 0; e < MAXE; ++e) {
        if (e < tt.ne) {
          // this step's increment in FP32, accumulated in FP64 (integrate_cell's arithmetic)
          LV v = LN::splat(ar.s[e]) * P;
#pragma unroll
          for (int l = 0; l <= N; ++l)
            if ((mask >> l) & 1u) v = fma(LN::splat(ar.c[e][l]), R[l], v);
          double* q = rb + e * ms;
          if constexpr (PPT == 2) {
            if (vk[0] && vk[1]) {
              double2 o = __ldcg(reinterpret_cast<const double2*>(q));
              o.x = fma(double(LN::get(v, 0)), ar.wfac, o.x);
              o.y = fma(double(LN::get(v, 1)), ar.wfac, o.y);
              *reinterpret_cast<double2*>(q) = o;
              continue;
            }
          }
#pragma unroll
          for (int k = 0; k < PPT; ++k)
            if (vk[k]) q[k] = fma(double(LN::get(v, k)), ar.wfac, __ldcg(q + k));
        }
      }
      if constexpr (C == 0) {
#pragma unroll
        for (int k = 0; k < PPT; ++k)
#pragma unroll
          for (int r = 0; r < MAXR; ++r)
            if (r < I.nr && vk[k]) I.wsum[(ce + k) * I.nr + r] = fma(ar.coef[r], double(own[lo + k]), wl[k][r]);
      }
    }
  }
  __syncthreads();   // the stage is reused by the next tile
}

template <int N, int DIMS>
__device__ __forceinline__ void tma_int_cell_of(const TILaunch<N>& L, const TTile& tt, unsigned char* st) {
  if constexpr (DIMS == 7) {
    switch (tt.cls) {
      case 0: tma_int_cell<N, 0, DIMS>(L, tt, st); break;
      case 1: tma_int_cell<N, 1, DIMS>(L, tt, st); break;
      case 2: tma_int_cell<N, 2, DIMS>(L, tt, st); break;
      case 3: tma_int_cell<N, 3, DIMS>(L, tt, st); break;
      case 4: tma_int_cell<N, 4, DIMS>(L, tt, st); break;
      case 5: tma_int_cell<N, 5, DIMS>(L, tt, st); break;
      case 6: tma_int_cell<N, 6, DIMS>(L, tt, st); break;
      default: tma_int_cell<N, 7, DIMS>(L, tt, st); break;
    }
  } else {
    switch (tt.cls) {
      case 0: tma_int_cell<N, 0, DIMS>(L, tt, st); break;
      case 2: tma_int_cell<N, 2, DIMS>(L, tt, st); break;
      case 4: tma_int_cell<N, 4, DIMS>(L, tt, st); break;
      default: tma_int_cell<N, 6, DIMS>(L, tt, st); break;
    }
  }
}

template <int N, int DIMS>
__global__ void __launch_bounds__(NTS, (TmaMinBlocks<N, DIMS>::value)) batch_tma_int_kernel(const __grid_constant__ TILaunch<N> L) {
  using LY = TmaIntLayout<N, DIMS>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long full[TSTAGES];
  if ((smem_u32(smem) & 127u) != 0u) {
    if (threadIdx.x == 0) atomicExch(L.status, (int)PN_ERR_INVALID);
    return;
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < TSTAGES; ++s) mbar_init(&full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int G = gridDim.x;
  const int t0 = blockIdx.x;
  if (threadIdx.x == 0)
    for (int k = 0; k < TSTAGES - 1; ++k) {
      const int t = t0 + k * G;
      if (t < L.n_tiles) tma_issue_int<N, DIMS>(L, L.tiles[t], smem + k * LY::STAGE, &full[k]);
    }
  for (int k = 0; t0 + k * G < L.n_tiles; ++k) {
    const int s = k % TSTAGES;
    const int ka = k + TSTAGES - 1;
    const int ta = t0 + ka * G;
    if (ta < L.n_tiles && threadIdx.x == 0) {
      bulk_wait_read();
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tma_issue_int<N, DIMS>(L, L.tiles[ta], smem + (ka % TSTAGES) * LY::STAGE, &full[ka % TSTAGES]);
    }
    const bool ok = mbar_wait_bounded(&full[s], (unsigned)((k / TSTAGES) & 1));
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(L.status, (int)PN_ERR_TIMEOUT);
        for (int kk = k; kk <= ka; ++kk)
          if (t0 + kk * G < L.n_tiles) mbar_wait_bounded(&full[kk % TSTAGES], (unsigned)((kk / TSTAGES) & 1));
        bulk_wait_all();
      }
      __syncthreads();
      return;
    }
    unsigned char* st = smem + s * LY::STAGE;
    const TTile& tt = *reinterpret_cast<const TTile*>(st + LY::TIL);
    tma_int_cell_of<N, DIMS>(L, tt, st);
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

}  // namespace pn

#include "pn_batch_par.cuh"   // 2D parity tiles (used by the sweep kernel below)

namespace pn {

// ---------------------------------------------------------------------------------------------
// one persistent launch per sweep
// ---------------------------------------------------------------------------------------------
// A sweep (a forward march, or an adjoint march with its density integrals and recomputed
// segments) is a sequence of steps; a step is what one launch of batch_tma_kernel or
// batch_tma_int_kernel covers.  batch_sweep_kernel runs every tile of every step in one
// cooperative launch: the tiles of all steps form one item list (step-major), which the CTAs walk
// in grid-stride order.  Before its loads, an item of solve q waits (bounded) until the last
// earlier step that had tiles of q has completed all of them (per-step, per-solve counters
// released after the tile's stores have landed).  A solve's steps therefore keep their order
// while the steps of different solves, and the end of one step and the start of the next,
// overlap.  Every CTA is resident (cooperative launch) and handles its items in increasing order,
// and every item waits only on items of earlier steps, so the CTA holding the lowest unfinished
// item can always proceed.
enum { TS_FWD = 0, TS_ADJ = 1, TS_INT = 2 };

struct TStep {
  int kind;       // TS_FWD / TS_ADJ sub-step (or fused pair), TS_INT density integral
  int list;       // tile list
  int mode, j, sub;
  int n_tiles;
  int first;      // index of the step's first item
  int pad_;
  double* partial;
};

template <int N>
struct TSweep {
  const BInst<float>* inst;
  const TSolve* solves;
  const TTile* tiles[3];
  const CUtensorMap* maps;
  const ArgRow<N>* rows;
  const IntRow<N>* irows;
  double* partial_unused_;
  int* status;
  int* test_expire;
  const TStep* steps;
  const int* dep;        // [step][solve]: the last earlier step with tiles of the solve, or -1
  const int* need;       // [step][solve]: tiles of the solve in that earlier step
  int* done;             // [step][solve]: tiles of the solve completed
  int n_steps, n_items, n_solves;
  int pr, K;
  int par;               // the sub-step lists hold parity tiles (2D)
};

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// release one completed tile of a sweep: its tensor stores have landed (bulk_wait_all), the
// generic writes of its threads (observed by thread 0 through the CTA barrier) are fenced, then
// the counter is incremented with release semantics
__device__ __forceinline__ void release_tile(int* counter, bool generic_writes) {
  bulk_wait_all();
  if (generic_writes) __threadfence();
  asm volatile("fence.proxy.async.global;" ::: "memory");
  asm volatile("red.release.gpu.global.add.s32 [%0], 1;" ::"l"(counter) : "memory");
}

// wait (at most ~1 s) until *p >= need
__device__ __forceinline__ bool wait_count(const int* p, int need) {
  if (ld_acquire(p) >= need) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (ld_acquire(p) >= need) return true;
    if (global_ns() - t0 > 1000000000ull) return false;
    __nanosleep(100);
  }
}

template <int N, int DIMS>
__global__ void __launch_bounds__(NTS, PN_TMA_MINB) batch_sweep_kernel(const __grid_constant__ TSweep<N> S) {
  static_assert(TSTAGES == 1, "the sweep kernel stages one tile per CTA");
  constexpr bool PAR_OK = DIMS == 3 && PPT == 1;   // 2D groups may use parity tiles (S.par)
  using LY = TmaLayout<N, DIMS>;
  using LI = TmaIntLayout<N, DIMS>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long full[1];
  __shared__ double red[NTS / 32][MAXR];
  __shared__ TLaunch<N> L;
  __shared__ TILaunch<N> IL;
  __shared__ int sh_kind;
  if ((smem_u32(smem) & 127u) != 0u) {
    if (threadIdx.x == 0) atomicExch(S.status, (int)PN_ERR_INVALID);
    return;
  }
  if (threadIdx.x == 0) {
    mbar_init(&full[0], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  int k = 0;   // step of the current item (items are visited in increasing order)
  unsigned phase = 0;
  // thread 0: the counter of the previous item, released once its stores have landed -- after the
  // next item's loads are issued (their latency covers the stores'), or before thread 0 blocks on
  // a dependency, so that a CTA never waits while holding a tile
  long long pend = -1;
  bool pend_generic = false;
  for (int w = blockIdx.x; w < S.n_items; w += gridDim.x) {
    bool ok = true;
    if (threadIdx.x == 0) {
      while (k + 1 < S.n_steps && S.steps[k + 1].first <= w) ++k;
      const TStep st = S.steps[k];
      const TTile* tl = S.tiles[st.list] + (w - st.first);
      const int q = tl->inst;
      const int d = S.dep[(long long)k * S.n_solves + q];
      if (d >= 0) {
        const int* cnt = S.done + (long long)d * S.n_solves + q;
        const int need = S.need[(long long)k * S.n_solves + q];
        if (ld_acquire(cnt) < need) {
          // about to block: release the tile this CTA still holds first, so that no two CTAs
          // can wait on each other's held tiles
          if (pend >= 0) {
            release_tile(S.done + pend, pend_generic);
            pend = -1;
          }
          ok = wait_count(cnt, need);
        }
        asm volatile("fence.proxy.async.global;" ::: "memory");
      }
      sh_kind = st.kind;
      if (st.kind == TS_INT) {
        IL.inst = S.inst;
        IL.solves = S.solves;
        IL.tiles = S.tiles[st.list];
        IL.maps = S.maps;
        IL.rows = S.irows;
        IL.status = S.status;
        IL.n_tiles = st.n_tiles;
        IL.it = st.j;
        IL.K = S.K;
      } else {
        L.inst = S.inst;
        L.solves = S.solves;
        L.tiles = S.tiles[st.list];
        L.maps = S.maps;
        L.rows = S.rows;
        L.partial = st.partial;
        L.status = S.status;
        L.test_expire = S.test_expire;
        L.pr = S.pr;
        L.n_tiles = st.n_tiles;
        L.mode = st.mode;
        L.j = st.j;
        L.K = S.K;
        L.sub = st.sub;
      }
      if (ok) {
        bulk_wait_read();   // the previous item's stores have read the stage
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (st.kind == TS_INT) tma_issue_int<N, DIMS>(IL, *tl, smem, &full[0]);
        else if (PAR_OK && S.par) {
          if constexpr (PAR_OK) {
            if (st.kind == TS_ADJ) par_issue<N, true>(L, *tl, smem, &full[0]);
            else par_issue<N, false>(L, *tl, smem, &full[0]);
          }
        } else if (st.kind == TS_ADJ) tma_issue<N, true, DIMS>(L, *tl, smem, &full[0]);
        else tma_issue<N, false, DIMS>(L, *tl, smem, &full[0]);
      }
    }
    if (__syncthreads_or(!ok)) {   // a dependency did not complete in time: nothing was issued
      if (threadIdx.x == 0) {
        atomicExch(S.status, (int)PN_ERR_TIMEOUT);
        bulk_wait_all();
      }
      __syncthreads();
      return;
    }
    ok = mbar_wait_bounded(&full[0], phase);
    if (threadIdx.x == 0 && ok && sh_kind != TS_INT && S.test_expire != nullptr && w == (int)blockIdx.x &&
        *(volatile int*)S.test_expire > 0 && atomicSub(S.test_expire, 1) > 0)
      ok = false;   // test hook: report the first (completed) wait as run out, as batch_tma_kernel does
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(S.status, (int)PN_ERR_TIMEOUT);
        mbar_wait_bounded(&full[0], phase);   // let the copies in flight land
        bulk_wait_all();
      }
      __syncthreads();
      return;
    }
    phase ^= 1u;
    if (threadIdx.x == 0 && pend >= 0) {
      release_tile(S.done + pend, pend_generic);
      pend = -1;
    }
    const int kind = sh_kind;
    if (kind == TS_INT) {
      const TTile& tt = *reinterpret_cast<const TTile*>(smem + LI::TIL);
      tma_int_cell_of<N, DIMS>(IL, tt, smem);
    } else if (PAR_OK && S.par) {
      if constexpr (PAR_OK) {
        const TTile& tt = *reinterpret_cast<const TTile*>(smem + ParLayout<N>::TIL);
        if (kind == TS_ADJ) par_tile<N, true>(L, tt, smem, red);
        else par_tile<N, false>(L, tt, smem, red);
      }
    } else {
      const TTile& tt = *reinterpret_cast<const TTile*>(smem + LY::TIL);
      if (kind == TS_ADJ) tma_cell_of<N, true, DIMS>(L, tt, smem, red);
      else tma_cell_of<N, false, DIMS>(L, tt, smem, red);
    }
    // the tile is released later (see pend): its tensor stores (sub-steps) or its rho_bar and
    // line sums (the integral's threads synchronised at its end) are then visible
    if (threadIdx.x == 0) {
      const int til = kind == TS_INT ? LI::TIL : (PAR_OK && S.par) ? ParLayout<N>::TIL : LY::TIL;
      const TTile& tt = *reinterpret_cast<const TTile*>(smem + til);
      pend = (long long)k * S.n_solves + tt.inst;
      pend_generic = kind == TS_INT;
    }
    __syncthreads();   // the stage's tile record is not read again before the next issue
  }
  if (threadIdx.x == 0) {
    if (pend >= 0) release_tile(S.done + pend, pend_generic);
    bulk_wait_all();
  }
}

// ---------------------------------------------------------------------------------------------
// host: tensor maps
// ---------------------------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    else
      cudaGetLastError();
  });
  return fn;
}

// tensor of rank 4 (x, y, z, moment) or 5 (x, y, z, moment, slot) of 4- or 8-byte floats; strides
// in elements
inline bool encode_tensor(CUtensorMap* out, void* base, int rank, const long long* dims, const long long* strides,
                          const int* box, int elem_bytes) {
  EncodeTiledFn fn = encode_tiled_fn();
  if (!fn || rank < 1 || rank > 5) return false;
  cuuint64_t gd[5], gs[4];
  cuuint32_t bd[5], es[5];
  for (int d = 0; d < rank; ++d) {
    gd[d] = (cuuint64_t)dims[d];
    bd[d] = (cuuint32_t)box[d];
    es[d] = 1;
    if (d > 0) gs[d - 1] = (cuuint64_t)strides[d] * (cuuint64_t)elem_bytes;
  }
  const CUtensorMapDataType dt = elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  return fn(out, dt, (cuuint32_t)rank, base, gd, gs, bd, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

inline bool encode_f32(CUtensorMap* out, void* base, int rank, const long long* dims, const long long* strides,
                       const int* box) {
  return encode_tensor(out, base, rank, dims, strides, box, 4);
}

}  // namespace pn
