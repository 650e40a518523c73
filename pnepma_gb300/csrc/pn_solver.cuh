// pn_solver.cuh -- one solve on one GPU: device memory, work segmentation, the forward march with
// its tape, the adjoint march, and the CUDA graphs that replay them.
//
// Energy-step structure (StaRMAP step_pde!, starmap/src/solver.jl:171-196): odd classes by dt/2,
// even classes by dt, odd classes by dt/2; each launch computes the boundary ghosts it needs.
// The forward tape is the state itself: step i reads slot i-1 and writes slot i, so no state is
// ever copied.  With a checkpoint stride K only every K-th state is kept and the adjoint sweep
// recomputes each segment from its checkpoint before walking it backwards.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "pn_device.cuh"
#include "pn_layout.h"
#include "pn_tape_pool.h"
#include "pn_solver_base.h"
#include "pn_util.cuh"

namespace pn {

// final intensities in step order: I_r = sum_i (((dE dvol) sigma_{i,r}) integral_{i,r}) w_i
static __global__ void final_intensity_kernel(const double* __restrict__ integral, const double* __restrict__ sigma,
                                       const double* __restrict__ weight, double* __restrict__ I, int ns1,
                                       int nr, double dE, double dvol, double inv_scale) {
  const int r = threadIdx.x;
  if (r >= nr) return;
  double acc = 0.0;
  for (int i = 0; i < ns1; ++i) acc = acc + dE * dvol * sigma[(long long)i * nr + r] * integral[(long long)i * nr + r] * weight[i];
  I[r] = acc * inv_scale;
}

#define PN_CUDA(call)                                                   \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) {                                            \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);         \
      return PN_ERR_CUDA;                                               \
    }                                                                   \
  } while (0)

inline int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152 * 16) b = 152 * 16;
  return (int)b;
}

// Descriptor checks shared by the handle path (pn_create) and the no-allocation forward
// (pn_forward_noalloc), so that both accept and reject the same descriptors: table limits, the
// grid limits of the cell packing (pack_cell keeps 11 bits of x and y and 10 of z), presence of
// the forward tables (and of the adjoint tables when `adjoint`), a positive energy step and cell
// volume, PN_FLAG_CHECK_CFL, the line-to-element map and positive, finite stopping powers.
inline int validate_desc(const pn_desc* d, const Layout& L, bool adjoint, std::string& err) {
  if (L.ne > MAXE) { err = "at most " + std::to_string(MAXE) + " elements per solve are supported"; return PN_ERR_UNSUPPORTED; }
  if (L.nr > MAXR) { err = "at most " + std::to_string(MAXR) + " x-ray lines per solve are supported"; return PN_ERR_UNSUPPORTED; }
  for (int k = 0; k < 3; ++k)
    if (L.M[k] > 2000 || (k == 2 && L.M[k] > 1000)) { err = "grid too large for the cell packing"; return PN_ERR_UNSUPPORTED; }
  if (!d->advection || !d->boundary_fwd || !d->beam_face || !d->fwd_s || !d->fwd_c || !d->fwd_bc || !d->fwd_sigma ||
      !d->fwd_weight || (L.nr > 0 && !d->xray_element)) {
    err = "descriptor has a NULL table";
    return PN_ERR_INVALID;
  }
  if (adjoint && (!d->boundary_adj || !d->adj_int_s || !d->adj_int_c || !d->adj_int_bc || !d->adj_sigma ||
                  !d->adj_weight || !d->adj_src_sigma || !d->adj_s || !d->adj_c)) {
    err = "descriptor has a NULL table";
    return PN_ERR_INVALID;
  }
  if (!(d->delta_e > 0.0) || !(d->dvol > 0.0)) { err = "delta_e and dvol must be positive"; return PN_ERR_INVALID; }
  if ((d->flags & PN_FLAG_CHECK_CFL) && d->delta_e > d->cfl_limit) {
    err = "energy step " + std::to_string(d->delta_e) + " exceeds cfl_limit " + std::to_string(d->cfl_limit);
    return PN_ERR_CFL;
  }
  for (int r = 0; r < L.nr; ++r)
    if (d->xray_element[r] < 0 || d->xray_element[r] >= L.ne) { err = "xray_element out of range"; return PN_ERR_INVALID; }
  const long long ns = L.ns, ne = L.ne;
  auto positive = [](double v) { return v > 0.0 && std::isfinite(v); };
  for (long long q = 0; q < ns * ne; ++q)
    if (!positive(d->fwd_s[q])) { err = "stopping power must be positive and finite"; return PN_ERR_INVALID; }
  if (adjoint) {
    for (long long q = 0; q < (ns + 1) * ne; ++q)
      if (!positive(d->adj_int_s[q])) { err = "stopping power must be positive and finite"; return PN_ERR_INVALID; }
    for (long long q = 0; q < ns * ne; ++q)
      if (!(d->adj_s[q] > 0.0)) { err = "stopping power must be positive and finite"; return PN_ERR_INVALID; }
  }
  return PN_OK;
}

// Advection values at the compiled stencil positions, divided by the grid step (tab[Ord<N>::n_tab]).
// Rejects blocks whose nonzero pattern differs from the compiled one: a zero at a stencil position
// or a nonzero outside it.
template <int N>
int advection_table(const pn_desc* d, const Layout& L, double* tab, std::string& err) {
  const double* pa = d->advection;
  int t = 0;
  std::vector<char> used;
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 8; ++c) {
      const int nrow = L.nm[c], ncol = L.nm[class_switch(c, k)];
      const int off = Ord<N>::off(c, k);
      // blocks are laid out class-major, axis-minor; this block ends where the next one starts
      const int endk = (c == 7 && k == 2) ? Ord<N>::n_tab : (k < 2 ? Ord<N>::off(c, k + 1) : Ord<N>::off(c + 1, 0));
      used.assign((size_t)nrow * ncol + 1, 0);
      for (int kk = off; kk < endk; ++kk) {
        const int row = Ord<N>::rc[kk][0], col = Ord<N>::rc[kk][1];
        const double v = pa[(long long)row * ncol + col];
        if (v == 0.0) { err = "advection block sparsity differs from the compiled stencil"; return PN_ERR_INVALID; }
        tab[kk] = v / d->h[k];
        used[(size_t)row * ncol + col] = 1;
        ++t;
      }
      for (int q = 0; q < nrow * ncol; ++q)
        if (!used[q] && pa[q] != 0.0) { err = "advection block sparsity differs from the compiled stencil"; return PN_ERR_INVALID; }
      pa += (long long)nrow * ncol;
    }
  if (t != Ord<N>::n_tab) { err = "internal: advection table size"; return PN_ERR_INVALID; }
  return PN_OK;
}

template <class T, int N>
class Solver : public SolverBase {
 public:
  Layout L;
  int K = 0;               // checkpoint stride (>= 1)
  int n_ck = 0, n_work = 0;
  double dE = 0, dvol = 0, h[3] = {1, 1, 1};
  double scale_g = 1.0;    // power-of-two multiplier of the beam source (FP32 only)
  double scale_i = 1.0;    // power-of-two multiplier of the cotangent (FP32 only)
  int flags = 0;
  std::vector<double> fwd_s, fwd_c, fwd_bc, fwd_sigma, fwd_weight;
  std::vector<double> adj_int_s, adj_int_c, adj_int_bc, adj_sigma, adj_weight, adj_src_sigma, adj_s, adj_c;
  std::vector<int> xel;
  std::vector<double> beam_face_h;
  double tab_h[Ord<N>::n_tab > 0 ? Ord<N>::n_tab : 1];

  // device memory
  std::vector<void*> allocs;
  long long bytes = 0;
  T* slots = nullptr;
  T* lam = nullptr;
  T* sstate = nullptr;      // state of the pn_step interface
  T* cache_d = nullptr;     // right-hand-side factors of the odd classes (see launch_substep)
  T* cache_cls[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  T* rho_d = nullptr;
  double* rbar_d = nullptr;
  double* noa_d = nullptr;
  double* acs_d = nullptr;
  double* wint_d = nullptr;
  double* ibar_d = nullptr;
  double* acs_bar_d = nullptr;
  double* noa_bar_d = nullptr;
  double* partial_d = nullptr;
  double* integral_d = nullptr;
  double* sigma_d = nullptr;
  double* weight_d = nullptr;
  double* I_d = nullptr;
  double* bf_d = nullptr;
  double* ba_d = nullptr;
  double* beam_d = nullptr;
  int* xel_d = nullptr;
  int* faces_d = nullptr;
  double* stage_d = nullptr;     // caller-layout staging, max(n_rho, n_state) doubles
  double* out_mul_d = nullptr;   // factor that undoes the FP32 scaling of the adjoint outputs
  int* flag_d = nullptr;
  const double* bmat_f[3][8] = {{nullptr}};
  const double* bmat_a[3][8] = {{nullptr}};
  const double* beam_p[8] = {nullptr};

  std::vector<Seg> segs_par[2];
  int nblk_par[2] = {0, 0};
  std::vector<Seg> segs_all;
  int nblk_all = 0;
  // ghost lines of the face cells, per parity of the target class (sub-steps) and all (integral)
  GLine* glines_d = nullptr;
  int gl_off[2] = {0, 0}, gl_n[2] = {0, 0};

  cudaStream_t stream = nullptr;
  // the even classes' density integral of an adjoint iteration runs on `side`, beside the odd
  // classes' integral and sub-step 1 (forked and joined by events inside the captured graph)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaGraphExec_t g_fwd = nullptr, g_adj = nullptr;
  bool have_forward = false;
  bool have_state = false;
  // full tape in the device's shared tape buffer (pn_tape_pool.h) instead of own checkpoints
  bool pool_user = false;
  int device = 0;
  unsigned long long hid = 0;          // this handle's id
  unsigned long long pool_epoch = 0;   // buffer address the graphs were captured with
  unsigned long long my_gen = 0;       // generation of this handle's last recorded tape

  ~Solver() override {
    if (g_fwd) cudaGraphExecDestroy(g_fwd);
    if (g_adj) cudaGraphExecDestroy(g_adj);
    if (pool_user) {
      TapePool& P = tape_pool(device);
      std::lock_guard<std::mutex> lk(P.mu);
      if (P.owner == hid) P.owner = 0;
      if (--P.users == 0 && P.base) {
        if (P.last) cudaEventSynchronize(P.last);
        cudaFree(P.base);
        P.base = nullptr;
        P.bytes = 0;
        ++P.epoch;
        P.owner = 0;
      }
    }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
    for (void* p : allocs) cudaFree(p);
  }

  // With the pool lock held: point `slots` at a buffer that holds this handle's full tape,
  // growing it if needed; re-capture the graphs when the address changed.  Returns false when
  // the tape does not fit (the handle then checkpoints with its own slots).
  bool pool_acquire(TapePool& P) {
    const size_t need = (size_t)(n_ck + n_work) * (size_t)L.slot_elems * sizeof(T);
    if (P.bytes < need) {
      if (P.base) {
        if (P.last) cudaEventSynchronize(P.last);
        cudaFree(P.base);
        P.base = nullptr;
        P.bytes = 0;
        ++P.epoch;
        P.owner = 0;
      }
      size_t fr = 0, tot = 0;
      if (cudaMemGetInfo(&fr, &tot) != cudaSuccess || need > fr / 10 * 8) {
        cudaGetLastError();
        return false;
      }
      void* q = nullptr;
      if (cudaMalloc(&q, need) != cudaSuccess) {
        cudaGetLastError();
        return false;
      }
      P.base = (char*)q;
      P.bytes = need;
      ++P.epoch;
      P.owner = 0;
    }
    if (!P.last && cudaEventCreateWithFlags(&P.last, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (pool_epoch != P.epoch) {
      slots = (T*)P.base;
      if (g_fwd) { cudaGraphExecDestroy(g_fwd); g_fwd = nullptr; }
      if (g_adj) { cudaGraphExecDestroy(g_adj); g_adj = nullptr; }
      pool_epoch = P.epoch;
    }
    return true;
  }

  // leave the pool for good: own checkpoints every ceil(sqrt(n_steps)) states
  int pool_leave(TapePool& P) {
    pool_user = false;
    --P.users;
    if (P.owner == hid) P.owner = 0;
    K = std::max(2, (int)std::ceil(std::sqrt((double)L.ns)));
    if (K > L.ns) K = L.ns;
    n_ck = L.ns / K + 1 + ((L.ns % K) ? 1 : 0);
    n_work = std::max(2, K - 1);
    if (g_fwd) { cudaGraphExecDestroy(g_fwd); g_fwd = nullptr; }
    if (g_adj) { cudaGraphExecDestroy(g_adj); g_adj = nullptr; }
    int rc;
    if ((rc = alloc(slots, (long long)(n_ck + n_work) * L.slot_elems))) return rc;
    return PN_OK;
  }

  long long device_bytes() const override { return bytes; }

  long long n_launch = 0;            // kernel launches recorded since the counter was reset
  long long fwd_kernels = 0, adj_kernels = 0;

  int n_active() const {
    int n = 0;
    for (int c = 0; c < 8; ++c) n += L.active[c] ? 1 : 0;
    return n;
  }

  void info(pn_handle_info* out) const override {
    out->checkpoint_stride = K;
    out->precision = sizeof(T) == 4 ? PN_FP32 : PN_FP64;
    out->device_bytes = bytes;
    // graph kernels + per-call layout kernels
    out->forward_kernels = fwd_kernels + n_active() + (L.nr ? 1 : 0);
    out->adjoint_kernels = adj_kernels + n_active() + 1 + (L.nr ? 2 : 1);
  }

  template <class U>
  int alloc(U*& p, long long n) {
    void* q = nullptr;
    size_t b = (size_t)std::max<long long>(n, 1) * sizeof(U);
    cudaError_t e = cudaMalloc(&q, b);
    if (e != cudaSuccess) {
      cudaGetLastError();
      err = "device allocation of " + std::to_string(b) + " bytes failed: " + cudaGetErrorString(e);
      return PN_ERR_NO_MEMORY;
    }
    allocs.push_back(q);
    bytes += (long long)b;
    p = (U*)q;
    return PN_OK;
  }

  T* slot(int idx) { return slots + (long long)idx * L.slot_elems; }
  int ck_index(int step) const { return (step == L.ns) ? n_ck - 1 : step / K; }
  bool is_ck(int step) const { return step % K == 0 || step == L.ns; }
  T* fwd_slot(int step) { return is_ck(step) ? slot(ck_index(step)) : slot(n_ck + (step % 2)); }

  // ------------------------------------------------------------------------------------------
  int create(const pn_desc* d) override {
    int rc = L.init(d, err);
    if (rc) return rc;
    if (L.N != N) { err = "internal: order mismatch"; return PN_ERR_INVALID; }
    if ((rc = validate_desc(d, L, true, err))) return rc;
    flags = d->flags;
    dE = d->delta_e;
    dvol = d->dvol;
    for (int k = 0; k < 3; ++k) h[k] = d->h[k];
    const int ns = L.ns, ne = L.ne, nr = L.nr, N1 = N + 1;
    auto cp = [](const double* p, long long n) { return std::vector<double>(p, p + n); };
    fwd_s = cp(d->fwd_s, (long long)ns * ne);
    fwd_c = cp(d->fwd_c, (long long)ns * ne * N1);
    fwd_bc = cp(d->fwd_bc, ns);
    fwd_sigma = cp(d->fwd_sigma, (long long)(ns + 1) * nr);
    fwd_weight = cp(d->fwd_weight, ns + 1);
    adj_int_s = cp(d->adj_int_s, (long long)(ns + 1) * ne);
    adj_int_c = cp(d->adj_int_c, (long long)(ns + 1) * ne * N1);
    adj_int_bc = cp(d->adj_int_bc, ns + 1);
    adj_sigma = cp(d->adj_sigma, (long long)(ns + 1) * nr);
    adj_weight = cp(d->adj_weight, ns + 1);
    adj_src_sigma = cp(d->adj_src_sigma, (long long)(ns + 1) * nr);
    adj_s = cp(d->adj_s, (long long)(ns + 1) * ne);
    adj_c = cp(d->adj_c, (long long)(ns + 1) * ne * N1);
    xel.assign(d->xray_element, d->xray_element + nr);
    beam_face_h = cp(d->beam_face, L.n_beam);
    if ((rc = advection_table<N>(d, L, tab_h, err))) return rc;

    // checkpoint stride
    const long long slot_bytes = L.slot_elems * (long long)sizeof(T);
    K = d->checkpoint_stride;
    if (K < 0) { err = "checkpoint_stride must be >= 0"; return PN_ERR_INVALID; }
    if (K == 0) {
      // a full tape up to 2 GiB of its own; beyond, a full tape in the device's shared buffer
      const long long budget = 2LL << 30;
      K = 1;
      if ((long long)(ns + 1) * slot_bytes > budget) pool_user = true;
    }
    if (K > ns) K = ns;
    n_ck = ns / K + 1 + ((ns % K) ? 1 : 0);
    n_work = std::max(2, K - 1);

    // scaling of the FP32 state (powers of two: exact)
    if (sizeof(T) == 4) {
      double gmax = 0.0, bmax = 0.0;
      for (double v : beam_face_h) gmax = std::max(gmax, std::fabs(v));
      for (double v : fwd_bc) bmax = std::max(bmax, std::fabs(v));
      for (double v : adj_int_bc) bmax = std::max(bmax, std::fabs(v));
      const double m = gmax * bmax;
      if (m > 0.0 && std::isfinite(m)) scale_g = std::ldexp(1.0, -(int)std::lround(std::log2(m)));
    }

    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming) != cudaSuccess) {
      err = "cudaStreamCreate / cudaEventCreate failed";
      return PN_ERR_CUDA;
    }
    // allocations (a pool user takes its tape from the shared buffer at its first forward)
    const int nslots = n_ck + n_work;
    PN_CUDA(cudaGetDevice(&device));
    hid = next_handle_id();
    if (pool_user) {
      TapePool& P = tape_pool(device);
      std::lock_guard<std::mutex> lk(P.mu);
      ++P.users;
    } else if ((rc = alloc(slots, (long long)nslots * L.slot_elems))) {
      return rc;
    }
    if ((rc = alloc(lam, L.slot_elems))) return rc;
    if ((rc = alloc(sstate, L.slot_elems))) return rc;
    if ((rc = alloc(rho_d, L.rho_elems))) return rc;
    if ((rc = alloc(rbar_d, L.rho_elems))) return rc;
    const long long ncell = L.n_eee_cells;
    if ((rc = alloc(noa_d, ncell * ne))) return rc;
    if ((rc = alloc(acs_d, ncell * std::max(nr, 1)))) return rc;
    if ((rc = alloc(wint_d, ncell * std::max(nr, 1)))) return rc;
    if ((rc = alloc(ibar_d, std::max(nr, 1)))) return rc;
    if ((rc = alloc(acs_bar_d, ncell * std::max(nr, 1)))) return rc;
    if ((rc = alloc(noa_bar_d, ncell * ne))) return rc;
    if ((rc = alloc(integral_d, (long long)(ns + 1) * std::max(nr, 1)))) return rc;
    if ((rc = alloc(sigma_d, (long long)(ns + 1) * std::max(nr, 1)))) return rc;
    if ((rc = alloc(weight_d, ns + 1))) return rc;
    if ((rc = alloc(I_d, std::max(nr, 1)))) return rc;
    if ((rc = alloc(bf_d, L.n_bnd))) return rc;
    if ((rc = alloc(ba_d, L.n_bnd))) return rc;
    if ((rc = alloc(beam_d, std::max<long long>(L.n_beam, 1)))) return rc;
    {
      // factor cache of the odd classes: planes C_0..C_N, g_0..g_N (g_l = dt phi1_l / S) with each
      // class's geometry
      long long n_cache = 0;
      for (int cl = 0; cl < 8; ++cl)
        if (L.active[cl] && class_parity(cl) == 1) n_cache += (long long)(2 * N + 2) * L.ms[cl];
      if (n_cache > 0) {
        if ((rc = alloc(cache_d, n_cache))) return rc;
        long long o = 0;
        for (int cl = 0; cl < 8; ++cl)
          if (L.active[cl] && class_parity(cl) == 1) {
            cache_cls[cl] = cache_d + o;
            o += (long long)(2 * N + 2) * L.ms[cl];
          }
      }
    }
    if ((rc = alloc(xel_d, std::max(nr, 1)))) return rc;
    if ((rc = alloc(stage_d, std::max(L.n_rho, L.n_state)))) return rc;
    if ((rc = alloc(flag_d, 1))) return rc;
    if ((rc = alloc(out_mul_d, 1))) return rc;
    if (!pool_user) PN_CUDA(cudaMemsetAsync(slots, 0, sizeof(T) * (size_t)nslots * L.slot_elems, stream));
    PN_CUDA(cudaMemsetAsync(sstate, 0, sizeof(T) * (size_t)L.slot_elems, stream));
    PN_CUDA(cudaMemsetAsync(rho_d, 0, sizeof(T) * (size_t)L.rho_elems, stream));
    PN_CUDA(cudaMemcpyAsync(bf_d, d->boundary_fwd, sizeof(double) * L.n_bnd, cudaMemcpyHostToDevice, stream));
    PN_CUDA(cudaMemcpyAsync(ba_d, d->boundary_adj, sizeof(double) * L.n_bnd, cudaMemcpyHostToDevice, stream));
    if (L.n_beam) PN_CUDA(cudaMemcpyAsync(beam_d, beam_face_h.data(), sizeof(double) * L.n_beam, cudaMemcpyHostToDevice, stream));
    if (nr) {
      PN_CUDA(cudaMemcpyAsync(xel_d, xel.data(), sizeof(int) * nr, cudaMemcpyHostToDevice, stream));
      PN_CUDA(cudaMemcpyAsync(sigma_d, fwd_sigma.data(), sizeof(double) * fwd_sigma.size(), cudaMemcpyHostToDevice, stream));
    }
    PN_CUDA(cudaMemcpyAsync(weight_d, fwd_weight.data(), sizeof(double) * fwd_weight.size(), cudaMemcpyHostToDevice, stream));
    {
      long long off = 0;
      for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 8; ++c)
          if (class_bit(c, k)) {
            bmat_f[k][c] = bf_d + off;
            bmat_a[k][c] = ba_d + off;
            off += (long long)L.nm[c] * L.nm[class_switch(c, k)];
          }
      for (int c = 4; c < 8; ++c) beam_p[c] = beam_d + L.beam_off[c];
    }
    if ((rc = build_segments())) return rc;
    PN_CUDA(cudaStreamSynchronize(stream));
    if (!pool_user) {
      if ((rc = capture(g_fwd, true))) return rc;
      if ((rc = capture(g_adj, false))) return rc;
    }
    return PN_OK;
  }

  // ------------------------------------------------------------------------------------------
  // work segmentation: inner boxes and face lists per target class
  int build_segments() {
    std::vector<int> all_faces;
    struct Tmp { int cls; int lo[3], ext[3]; long long face_off; int n_face; };
    std::vector<Tmp> per_class;
    for (int c = 0; c < 8; ++c) {
      if (!L.active[c]) continue;
      Tmp t{};
      t.cls = c;
      int ilo[3], ihi[3], blo[3], bhi[3];
      for (int k = 0; k < 3; ++k) {
        const int n = L.shape[c][k];
        if (!L.act[k]) { ilo[k] = 0; ihi[k] = 1; blo[k] = 0; bhi[k] = 1; }
        else if (class_bit(c, k)) { ilo[k] = 1; ihi[k] = n - 1; blo[k] = 1; bhi[k] = n - 1; }
        else { ilo[k] = 0; ihi[k] = n; blo[k] = 1; bhi[k] = n - 1; }
        t.lo[k] = blo[k];
        t.ext[k] = std::max(0, bhi[k] - blo[k]);
      }
      t.face_off = (long long)all_faces.size();
      for (int kz = ilo[2]; kz < ihi[2]; ++kz)
        for (int jy = ilo[1]; jy < ihi[1]; ++jy)
          for (int ix = ilo[0]; ix < ihi[0]; ++ix) {
            const int cc[3] = {ix, jy, kz};
            bool face = false;
            for (int k = 0; k < 3; ++k)
              if (L.act[k] && !class_bit(c, k) && (cc[k] == 0 || cc[k] == L.shape[c][k] - 1)) face = true;
            if (face) all_faces.push_back(pack_cell(ix, jy, kz));
          }
      t.n_face = (int)((long long)all_faces.size() - t.face_off);
      per_class.push_back(t);
    }
    int rc;
    // ghost lines in ghosts_for_cell's order per face cell: parity 0's, then parity 1's (the
    // integral of every class takes both ranges, which are adjacent)
    std::vector<GLine> lines;
    for (int par = 0; par < 2; ++par) {
      gl_off[par] = (int)lines.size();
      for (const Tmp& t : per_class) {
        if (class_parity(t.cls) != par) continue;
        for (int f = 0; f < t.n_face; ++f) {
          const int cell = all_faces[(size_t)t.face_off + f];
          const int cc[3] = {cell & 2047, (cell >> 11) & 2047, (cell >> 22) & 1023};
          for (int k = 0; k < 3; ++k) {
            if (!L.act[k] || class_bit(t.cls, k)) continue;
            if (cc[k] == 0) lines.push_back(GLine{t.cls, k, 1, cell});
            if (cc[k] == L.shape[t.cls][k] - 1) lines.push_back(GLine{t.cls, k, 0, cell});
          }
        }
      }
      gl_n[par] = (int)lines.size() - gl_off[par];
    }
    if ((rc = alloc(glines_d, (long long)std::max<size_t>(lines.size(), 1)))) return rc;
    if (!lines.empty())
      PN_CUDA(cudaMemcpyAsync(glines_d, lines.data(), sizeof(GLine) * lines.size(), cudaMemcpyHostToDevice, stream));
    // `lines` is pageable host memory: staged before the copy call returns
    if ((rc = alloc(faces_d, (long long)std::max<size_t>(all_faces.size(), 1)))) return rc;
    if (!all_faces.empty())
      PN_CUDA(cudaMemcpyAsync(faces_d, all_faces.data(), sizeof(int) * all_faces.size(), cudaMemcpyHostToDevice, stream));
    auto add = [&](std::vector<Seg>& segs, int& nblk, const Tmp& t) {
      if (t.ext[0] > 0 && t.ext[1] > 0 && t.ext[2] > 0) {
        Seg s{};
        s.cls = t.cls;
        s.kind = 0;
        s.block0 = nblk;
        for (int k = 0; k < 3; ++k) { s.lo[k] = t.lo[k]; s.ext[k] = t.ext[k]; }
        s.tile_x = (t.ext[1] > 1 || t.ext[2] > 1) ? 32 : PBLOCK;
        s.tiles_x = (t.ext[0] + s.tile_x - 1) / s.tile_x;
        const int ty = PBLOCK / s.tile_x;
        s.tiles_y = (t.ext[1] + ty - 1) / ty;
        s.nblocks = s.tiles_x * s.tiles_y * t.ext[2];
        nblk += s.nblocks;
        segs.push_back(s);
      }
      if (t.n_face > 0) {
        Seg s{};
        s.cls = t.cls;
        s.kind = 1;
        s.block0 = nblk;
        s.tile_x = PBLOCK;
        s.tiles_x = s.tiles_y = 1;
        s.n_face = t.n_face;
        s.faces = faces_d + t.face_off;
        s.nblocks = (t.n_face + PBLOCK - 1) / PBLOCK;
        nblk += s.nblocks;
        segs.push_back(s);
      }
    };
    for (const Tmp& t : per_class) {
      add(segs_par[class_parity(t.cls)], nblk_par[class_parity(t.cls)], t);
      add(segs_all, nblk_all, t);
    }
    if ((int)segs_par[0].size() > MAXSEG || (int)segs_par[1].size() > MAXSEG || (int)segs_all.size() > MAXSEG) {
      err = "internal: too many work segments";
      return PN_ERR_INVALID;
    }
    if (nblk_par[0] == 0 || nblk_par[1] == 0) { err = "grid too small: a parity has no cells"; return PN_ERR_INVALID; }
    int rc2;
    if ((rc2 = alloc(partial_d, (long long)(L.ns + 1) * nblk_par[0] * std::max(L.nr, 1)))) return rc2;
    return PN_OK;
  }

  // ------------------------------------------------------------------------------------------
  // launch builders
  void common_geom(Geom* g) {
    for (int c = 0; c < 8; ++c) {
      Geom q{};
      if (L.active[c]) {
        for (int k = 0; k < 3; ++k) q.n[k] = L.shape[c][k];
        q.px = L.px[c];
        q.nm = L.nm[c];
        q.ms = L.ms[c];
      }
      g[c] = q;
    }
  }

  // the ghosts of the face cells of lines [off, off + n) on stream st (see ghost_kernel)
  int launch_ghosts(T* const* rd, bool adj, double bc, int off, int n, cudaStream_t st) {
    if (n <= 0) return PN_OK;
    GhostArgs<T> g;
    std::memset(&g, 0, sizeof(g));
    common_geom(g.g);
    for (int cl = 0; cl < 8; ++cl) {
      g.rd[cl] = rd[cl];
      for (int k = 0; k < 3; ++k) g.bmat[k][cl] = adj ? bmat_a[k][cl] : bmat_f[k][cl];
      g.beam[cl] = beam_p[cl];
    }
    g.bc_scaled = bc * scale_g;
    g.source = adj ? 0 : 1;
    g.lines = glines_d + off;
    g.n_lines = n;
    ghost_kernel<T, N><<<(n * 32 + 255) / 256, 256, 0, st>>>(g);
    PN_CUDA(cudaGetLastError());
    ++n_launch;
    return PN_OK;
  }

  // one sub-step for the classes of parity `par`; own_rd/own_wr are the target slot pointers, from_rd
  // the slot holding the other parity
  int launch_substep(int par, bool adj, double dt, const double* s, const double* c, double bc, T* own_rd,
                     T* own_wr, T* from_rd, double* partial, const double* sig_src, int cache_mode = 0) {
    SubArgs<T, N> a;
    std::memset(&a, 0, sizeof(a));
    common_geom(a.g);
    for (int cl = 0; cl < 8; ++cl) {
      if (!L.active[cl]) continue;
      const bool tgt = class_parity(cl) == par;
      a.rd[cl] = (tgt ? own_rd : from_rd) + L.dev_off[cl];
      a.wr[cl] = tgt ? own_wr + L.dev_off[cl] : nullptr;
      a.rho[cl] = rho_d + L.rho_off[cl];
      for (int k = 0; k < 3; ++k) a.bmat[k][cl] = adj ? bmat_a[k][cl] : bmat_f[k][cl];
      a.beam[cl] = beam_p[cl];
    }
    for (int k = 0; k < 3; ++k) a.act[k] = L.act[k];
    a.ne = L.ne;
    a.nr = L.nr;
    a.nseg = (int)segs_par[par].size();
    for (int q = 0; q < a.nseg; ++q) a.seg[q] = segs_par[par][q];
    a.dt = T(dt);
    a.bc = bc;
    a.scale_g = scale_g;
    for (int e = 0; e < L.ne; ++e) {
      a.s[e] = T(s[e]);
      for (int l = 0; l <= N; ++l) a.c[e][l] = T(c[e * (N + 1) + l]);
    }
    for (int e = L.ne; e < MAXE; ++e) a.s[e] = T(0);
    a.acs = acs_d;
    a.noa = noa_d;
    a.ibar = ibar_d;
    for (int r = 0; r < L.nr; ++r) {
      a.xel[r] = xel[r];
      a.sig_src[r] = sig_src ? sig_src[r] : 0.0;
    }
    a.adjoint_source = (adj && sig_src != nullptr) ? 1 : 0;
    a.wint = wint_d;
    a.partial = partial;
    a.cache_mode = (par == 1 && cache_d != nullptr) ? cache_mode : 0;
    for (int cl = 0; cl < 8; ++cl) a.cache[cl] = cache_cls[cl];
    for (int q = 0; q < Ord<N>::n_tab; ++q) a.tab[q] = T(tab_h[q]);
    int rc;
    if ((rc = launch_ghosts(a.rd, adj, bc, gl_off[par], gl_n[par], stream))) return rc;
    a.pre_ghosts = 1;
    const int nb = nblk_par[par];
    // two threads per cell (substep_split_kernel): the same segments, 2 x PBLOCK threads a block
    if (adj)
      substep_split_kernel<T, N, true><<<nb, 2 * PBLOCK, 0, stream>>>(a);
    else
      substep_split_kernel<T, N, false><<<nb, 2 * PBLOCK, 0, stream>>>(a);
    PN_CUDA(cudaGetLastError());
    ++n_launch;
    return PN_OK;
  }

  // density integral of adjoint iteration j on tape state u: every class (par < 0) or the classes
  // of one parity, on stream st (the handle's stream by default)
  int launch_integrate(int j, T* u, int par = -1, cudaStream_t st = nullptr) {
    IntArgs<T, N> a;
    std::memset(&a, 0, sizeof(a));
    common_geom(a.g);
    for (int cl = 0; cl < 8; ++cl) {
      if (!L.active[cl]) continue;
      a.u[cl] = u + L.dev_off[cl];
      a.lam[cl] = lam + L.dev_off[cl];
      a.rho[cl] = rho_d + L.rho_off[cl];
      a.rbar[cl] = rbar_d + L.rho_off[cl];
      for (int k = 0; k < 3; ++k) a.bmat[k][cl] = bmat_f[k][cl];
      a.beam[cl] = beam_p[cl];
    }
    for (int k = 0; k < 3; ++k) a.act[k] = L.act[k];
    a.ne = L.ne;
    a.nr = L.nr;
    const std::vector<Seg>& sg = par < 0 ? segs_all : segs_par[par];
    a.nseg = (int)sg.size();
    for (int q = 0; q < a.nseg; ++q) a.seg[q] = sg[q];
    a.bc = adj_int_bc[j];
    a.scale_g = scale_g;
    a.wfac = dvol * dE * adj_weight[j];
    const int N1 = N + 1;
    for (int e = 0; e < L.ne; ++e) {
      a.s[e] = T(adj_int_s[(long long)j * L.ne + e]);
      for (int l = 0; l <= N; ++l) a.c[e][l] = T(adj_int_c[((long long)j * L.ne + e) * N1 + l]);
    }
    a.acs = acs_d;
    a.noa = noa_d;
    a.ibar = ibar_d;
    a.acs_bar = acs_bar_d;
    a.noa_bar = noa_bar_d;
    for (int r = 0; r < L.nr; ++r) {
      a.xel[r] = xel[r];
      a.coef[r] = dE * dvol * adj_sigma[(long long)j * L.nr + r] * adj_weight[j];
    }
    for (int q = 0; q < Ord<N>::n_tab; ++q) a.tab[q] = T(tab_h[q]);
    // the integral forms the forward problem's ghosts on the tape state
    int rc;
    const int goff = par < 0 ? 0 : gl_off[par];
    const int gn = par < 0 ? gl_n[0] + gl_n[1] : gl_n[par];
    if ((rc = launch_ghosts(a.u, false, a.bc, goff, gn, st ? st : stream))) return rc;
    a.pre_ghosts = 1;
    integrate_split_kernel<T, N><<<par < 0 ? nblk_all : nblk_par[par], 2 * PBLOCK, 0, st ? st : stream>>>(a);
    PN_CUDA(cudaGetLastError());
    ++n_launch;
    return PN_OK;
  }

  // forward step `i` (1-based) from src into dst; partials of the intensity integral optional
  int forward_step(int i, T* src, T* dst, bool with_partial) {
    const int N1 = N + 1;
    const double* s = fwd_s.data() + (long long)(i - 1) * L.ne;
    const double* c = fwd_c.data() + (long long)(i - 1) * L.ne * N1;
    const double bc = fwd_bc[i - 1];
    const double dt2 = dE / 2;
    int rc;
    // the two half sub-steps share coefficients, densities and dt: the first stores the
    // right-hand-side factors of the odd classes, the second loads them
    if ((rc = launch_substep(1, false, dt2, s, c, bc, src, dst, src, nullptr, nullptr, 1))) return rc;
    double* part = with_partial ? partial_d + (long long)i * nblk_par[0] * L.nr : nullptr;
    if ((rc = launch_substep(0, false, dE, s, c, bc, src, dst, dst, part, nullptr))) return rc;
    if ((rc = launch_substep(1, false, dt2, s, c, bc, dst, dst, dst, nullptr, nullptr, 2))) return rc;
    return PN_OK;
  }

  // adjoint step j; sub-step 2 first waits for `before_even` and is followed by a record of
  // `after_even`, when given
  int adjoint_step(int j, cudaEvent_t before_even = nullptr, cudaEvent_t after_even = nullptr) {
    const int N1 = N + 1;
    const double* s = adj_s.data() + (long long)j * L.ne;
    const double* c = adj_c.data() + (long long)j * L.ne * N1;
    const double* sg = adj_src_sigma.data() + (long long)j * L.nr;
    const double dt2 = dE / 2;
    int rc;
    if ((rc = launch_substep(1, true, dt2, s, c, 0.0, lam, lam, lam, nullptr, sg, 1))) return rc;
    if (before_even) PN_CUDA(cudaStreamWaitEvent(stream, before_even, 0));
    if ((rc = launch_substep(0, true, dE, s, c, 0.0, lam, lam, lam, nullptr, sg))) return rc;
    if (after_even) PN_CUDA(cudaEventRecord(after_even, stream));
    if ((rc = launch_substep(1, true, dt2, s, c, 0.0, lam, lam, lam, nullptr, sg, 2))) return rc;
    return PN_OK;
  }

  // ------------------------------------------------------------------------------------------
  int record_forward() {
    int rc;
    PN_CUDA(cudaMemsetAsync(slot(0), 0, sizeof(T) * (size_t)L.slot_elems, stream));
    if (L.nr) PN_CUDA(cudaMemsetAsync(integral_d, 0, sizeof(double) * (size_t)(L.ns + 1) * L.nr, stream));
    for (int i = 1; i <= L.ns; ++i)
      if ((rc = forward_step(i, fwd_slot(i - 1), fwd_slot(i), L.nr > 0))) return rc;
    if (L.nr) {
      reduce_partials_kernel<<<L.ns, 256, 0, stream>>>(partial_d, integral_d, nblk_par[0], L.nr, 1);
      PN_CUDA(cudaGetLastError());
      final_intensity_kernel<<<1, 32, 0, stream>>>(integral_d, sigma_d, weight_d, I_d, L.ns + 1, L.nr, dE, dvol,
                                                   1.0 / scale_g);
      PN_CUDA(cudaGetLastError());
      n_launch += 2;
    }
    return PN_OK;
  }

  int record_adjoint() {
    int rc;
    PN_CUDA(cudaMemsetAsync(lam, 0, sizeof(T) * (size_t)L.slot_elems, stream));
    PN_CUDA(cudaMemsetAsync(rbar_d, 0, sizeof(double) * (size_t)L.rho_elems, stream));
    PN_CUDA(cudaMemsetAsync(acs_bar_d, 0, sizeof(double) * (size_t)L.n_eee_cells * std::max(L.nr, 1), stream));
    PN_CUDA(cudaMemsetAsync(noa_bar_d, 0, sizeof(double) * (size_t)L.n_eee_cells * L.ne, stream));
    int j = 0;
    const bool early = K == 1;   // every state kept: no recomputation between iterations
    for (int i = L.ns; i >= 1;) {
      // segment (a, b] holding step i
      const int a = ((i - 1) / K) * K;
      const int b = std::min(a + K, L.ns);
      // recompute a+1 .. b-1 into work slots
      for (int t = a + 1; t <= b - 1; ++t) {
        T* src = (t - 1 == a) ? slot(ck_index(a)) : slot(n_ck + (t - a - 2));
        T* dst = slot(n_ck + (t - a - 1));
        if ((rc = forward_step(t, src, dst, false))) return rc;
      }
      for (; i > a; --i, ++j) {
        T* u = (i == b) ? slot(ck_index(b)) : slot(n_ck + (i - a - 1));
        // The even classes' integral reads only the even adjoint classes (changed by sub-step 2)
        // and writes their rho_bar, acs_bar and noa_bar (eee cells) and the odd classes' ghost
        // points of the tape state; the odd classes' integral and sub-step 1 touch none of these.
        // So it runs on the side stream, joined before sub-step 2 (and so before any
        // recomputation reuses a slot).  With every state kept (no recomputation) it is forked
        // right after the previous iteration's sub-step 2, the last change of the even classes,
        // and so also overlaps that iteration's sub-step 3.
        const bool forked = early && j > 0;
        if (!forked) PN_CUDA(cudaEventRecord(ev_fork, stream));
        PN_CUDA(cudaStreamWaitEvent(side, ev_fork, 0));
        if ((rc = launch_integrate(j, u, 0, side))) return rc;
        PN_CUDA(cudaEventRecord(ev_join, side));
        if ((rc = launch_integrate(j, u, 1))) return rc;
        if ((rc = adjoint_step(j, ev_join, early && j + 1 < L.ns ? ev_fork : nullptr))) return rc;
      }
    }
    if ((rc = launch_integrate(L.ns, slot(ck_index(0))))) return rc;
    return PN_OK;
  }

  int capture(cudaGraphExec_t& exec, bool fwd) {
    cudaGraph_t graph = nullptr;
    n_launch = 0;
    PN_CUDA(cudaStreamSynchronize(stream));   // no earlier work pending on the capture stream
    PN_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = fwd ? record_forward() : record_adjoint();
    cudaError_t e = cudaStreamEndCapture(stream, &graph);
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
    (fwd ? fwd_kernels : adj_kernels) = n_launch;
    if (e != cudaSuccess) {
      err = std::string("graph instantiate: ") + cudaGetErrorString(e);
      return PN_ERR_CUDA;
    }
    return PN_OK;
  }

  // ------------------------------------------------------------------------------------------
  int load_rho(const double* rho, bool dev, cudaStream_t st) {
    const double* src = rho;
    if (!dev) {
      PN_CUDA(cudaMemcpyAsync(stage_d, rho, sizeof(double) * (size_t)L.n_rho, cudaMemcpyHostToDevice, st));
      src = stage_d;
    }
    for (int c = 0; c < 8; ++c) {
      if (!L.active[c]) continue;
      const long long n = L.npts[c] * L.ne;
      unpack_points_kernel<T><<<grid_for(n), 256, 0, st>>>(src + L.off_rho[c], rho_d + L.rho_off[c], L.shape[c][0],
                                                          L.shape[c][1], L.shape[c][2], L.px[c], L.ne, L.ms[c], 1.0);
      PN_CUDA(cudaGetLastError());
    }
    return PN_OK;
  }

  // The forward graph on stream s; a pool user records its tape into the shared buffer after the
  // previous user of the buffer is done with it.
  int launch_forward_graph(cudaStream_t s) {
    int rc;
    if (pool_user) {
      TapePool& P = tape_pool(device);
      std::unique_lock<std::mutex> lk(P.mu);
      if (!pool_acquire(P)) {
        if ((rc = pool_leave(P))) return rc;
      } else {
        if (!g_fwd && (rc = capture(g_fwd, true))) return rc;
        PN_CUDA(cudaStreamWaitEvent(s, P.last, 0));
        P.owner = hid;
        my_gen = ++P.gen;
        PN_CUDA(cudaGraphLaunch(g_fwd, s));
        PN_CUDA(cudaEventRecord(P.last, s));
        return PN_OK;
      }
    }
    if (!g_fwd && (rc = capture(g_fwd, true))) return rc;
    PN_CUDA(cudaGraphLaunch(g_fwd, s));
    return PN_OK;
  }

  // The adjoint graph on stream s; a pool user whose tape was overwritten by another handle (or
  // lost when the buffer grew) first records it again with its forward graph.
  int launch_adjoint_graph(cudaStream_t s) {
    int rc;
    if (pool_user) {
      TapePool& P = tape_pool(device);
      std::unique_lock<std::mutex> lk(P.mu);
      if (!pool_acquire(P)) {
        if ((rc = pool_leave(P))) return rc;
        lk.unlock();
        if ((rc = launch_forward_graph(s))) return rc;
      } else {
        if (!g_fwd && (rc = capture(g_fwd, true))) return rc;
        if (!g_adj && (rc = capture(g_adj, false))) return rc;
        PN_CUDA(cudaStreamWaitEvent(s, P.last, 0));
        if (P.owner != hid || P.gen != my_gen) {
          P.owner = hid;
          my_gen = ++P.gen;
          PN_CUDA(cudaGraphLaunch(g_fwd, s));
        }
        PN_CUDA(cudaGraphLaunch(g_adj, s));
        PN_CUDA(cudaEventRecord(P.last, s));
        return PN_OK;
      }
    }
    if (!g_adj && (rc = capture(g_adj, false))) return rc;
    PN_CUDA(cudaGraphLaunch(g_adj, s));
    return PN_OK;
  }

  int forward(const double* rho, const double* noa, const double* acs, double* I, cudaStream_t st,
              bool dev) override {
    int rc;
    if (!rho || !noa || !acs || (L.nr && !I)) { err = "NULL buffer"; return PN_ERR_INVALID; }
    cudaStream_t s = st ? st : stream;
    if ((rc = load_rho(rho, dev, s))) return rc;
    const long long ncell = L.n_eee_cells;
    const cudaMemcpyKind kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    PN_CUDA(cudaMemcpyAsync(noa_d, noa, sizeof(double) * (size_t)(ncell * L.ne), kind, s));
    if (L.nr) {
      PN_CUDA(cudaMemcpyAsync(acs_d, acs, sizeof(double) * (size_t)(ncell * L.nr), kind, s));
      wint_kernel<<<grid_for(ncell * L.nr), 256, 0, s>>>(acs_d, noa_d, xel_d, wint_d, ncell, L.nr, L.ne);
      PN_CUDA(cudaGetLastError());
    }
    if ((rc = launch_forward_graph(s))) return rc;
    if (L.nr) {
      PN_CUDA(cudaMemcpyAsync(I, I_d, sizeof(double) * L.nr, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    }
    if (!dev || (flags & PN_FLAG_CHECK_FINITE)) PN_CUDA(cudaStreamSynchronize(s));
    have_forward = true;
    if ((flags & PN_FLAG_CHECK_FINITE) && L.nr) {
      double hI[MAXR];
      PN_CUDA(cudaMemcpy(hI, I_d, sizeof(double) * L.nr, cudaMemcpyDeviceToHost));
      for (int r = 0; r < L.nr; ++r)
        if (!std::isfinite(hI[r])) { err = "intensities are not finite: the march diverged"; return PN_ERR_DIVERGED; }
    }
    return PN_OK;
  }

  int adjoint(const double* ibar, double* rho_bar, double* noa_bar, double* acs_bar, cudaStream_t st,
              bool dev) override {
    int rc;
    if (!have_forward) { err = "pn_adjoint needs a preceding pn_forward on this handle"; return PN_ERR_STATE; }
    if ((L.nr && !ibar) || !rho_bar || !noa_bar || (L.nr && !acs_bar)) { err = "NULL buffer"; return PN_ERR_INVALID; }
    cudaStream_t s = st ? st : stream;
    double* mul_d = out_mul_d;
    if (L.nr) {
      const double* src = ibar;
      if (!dev) {
        PN_CUDA(cudaMemcpyAsync(stage_d, ibar, sizeof(double) * L.nr, cudaMemcpyHostToDevice, s));
        src = stage_d;
      }
      double smax = 0.0;
      for (double v : adj_src_sigma) smax = std::max(smax, std::fabs(v));
      // the cotangent enters the adjoint source with sigma * ACS * NOA (ACS <= 1, NOA ~ 1e23)
      prep_ibar_kernel<<<1, 32, 0, s>>>(src, ibar_d, mul_d, L.nr, smax * 1e23, sizeof(T) == 4 ? 1 : 0, scale_g);
      PN_CUDA(cudaGetLastError());
    } else {
      const double one = 1.0 / scale_g;
      PN_CUDA(cudaMemcpyAsync(mul_d, &one, sizeof(double), cudaMemcpyHostToDevice, s));
    }
    if ((rc = launch_adjoint_graph(s))) return rc;
    // rho_bar to the caller layout (zeros on ghost points and inactive classes)
    PN_CUDA(cudaMemsetAsync(stage_d, 0, sizeof(double) * (size_t)L.n_rho, s));
    for (int c = 0; c < 8; ++c) {
      if (!L.active[c]) continue;
      const long long n = L.npts[c] * L.ne;
      pack_points_kernel<double><<<grid_for(n), 256, 0, s>>>(rbar_d + L.rho_off[c], stage_d + L.off_rho[c],
                                                              L.shape[c][0], L.shape[c][1], L.shape[c][2], L.px[c],
                                                              L.ne, L.ms[c], 1.0, 0, 0, 0, 0, 0, 0, 0, mul_d);
      PN_CUDA(cudaGetLastError());
    }
    const long long ncell = L.n_eee_cells;
    scale_kernel<<<grid_for(ncell * L.ne), 256, 0, s>>>(noa_bar_d, ncell * L.ne, 1.0, mul_d);
    if (L.nr) scale_kernel<<<grid_for(ncell * L.nr), 256, 0, s>>>(acs_bar_d, ncell * L.nr, 1.0, mul_d);
    PN_CUDA(cudaGetLastError());
    const cudaMemcpyKind kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    PN_CUDA(cudaMemcpyAsync(rho_bar, stage_d, sizeof(double) * (size_t)L.n_rho, kind, s));
    PN_CUDA(cudaMemcpyAsync(noa_bar, noa_bar_d, sizeof(double) * (size_t)(ncell * L.ne), kind, s));
    if (L.nr) PN_CUDA(cudaMemcpyAsync(acs_bar, acs_bar_d, sizeof(double) * (size_t)(ncell * L.nr), kind, s));
    if (!dev) PN_CUDA(cudaStreamSynchronize(s));
    return PN_OK;
  }

  int generation_field(const double* rho, double* field) override {
    int rc;
    if (!rho || (L.nr && !field)) { err = "NULL buffer"; return PN_ERR_INVALID; }
    if ((rc = load_rho(rho, false, stream))) return rc;
    double* f_d = nullptr;
    const long long ncell = L.n_eee_cells;
    // the acs_bar buffer has the right size for the field ([cell][r])
    f_d = acs_bar_d;
    PN_CUDA(cudaMemsetAsync(f_d, 0, sizeof(double) * (size_t)ncell * std::max(L.nr, 1), stream));
    PN_CUDA(cudaMemsetAsync(sstate, 0, sizeof(T) * (size_t)L.slot_elems, stream));
    for (int i = 1; i <= L.ns; ++i) {
      if ((rc = forward_step(i, sstate, sstate, false))) return rc;
      if (L.nr) {
        generation_kernel<T><<<grid_for(ncell), 256, 0, stream>>>(sstate + L.dev_off[0], f_d, L.shape[0][0],
                                                                  L.shape[0][1], L.shape[0][2], L.px[0], L.nr, dE,
                                                                  sigma_d + (long long)i * L.nr, fwd_weight[i],
                                                                  1.0 / scale_g);
        PN_CUDA(cudaGetLastError());
      }
    }
    if (L.nr) PN_CUDA(cudaMemcpyAsync(field, f_d, sizeof(double) * (size_t)(ncell * L.nr), cudaMemcpyDeviceToHost, stream));
    PN_CUDA(cudaStreamSynchronize(stream));
    have_state = false;
    return PN_OK;
  }

  int set_state(const double* rho, const double* state) override {
    int rc;
    if (!rho || !state) { err = "NULL buffer"; return PN_ERR_INVALID; }
    if ((rc = load_rho(rho, false, stream))) return rc;
    PN_CUDA(cudaMemcpyAsync(stage_d, state, sizeof(double) * (size_t)L.n_state, cudaMemcpyHostToDevice, stream));
    PN_CUDA(cudaMemsetAsync(sstate, 0, sizeof(T) * (size_t)L.slot_elems, stream));
    for (int c = 0; c < 8; ++c) {
      if (!L.active[c] || L.nm[c] == 0) continue;
      const long long n = L.npts[c] * L.nm[c];
      // the FP32 state is kept in units of the scaled source (a power of two: exact)
      unpack_points_kernel<T><<<grid_for(n), 256, 0, stream>>>(stage_d + L.off_state[c], sstate + L.dev_off[c],
                                                              L.shape[c][0], L.shape[c][1], L.shape[c][2], L.px[c],
                                                              L.nm[c], L.ms[c], scale_g);
      PN_CUDA(cudaGetLastError());
    }
    PN_CUDA(cudaStreamSynchronize(stream));
    have_state = true;
    return PN_OK;
  }

  int step(int i) override {
    int rc;
    if (!have_state) { err = "pn_step needs pn_set_state first"; return PN_ERR_STATE; }
    if (i < 0 || i >= L.ns) { err = "step index out of range"; return PN_ERR_INVALID; }
    if ((rc = forward_step(i + 1, sstate, sstate, false))) return rc;
    PN_CUDA(cudaStreamSynchronize(stream));
    return PN_OK;
  }

  int get_state(double* state) override {
    if (!have_state) { err = "no state: call pn_set_state first"; return PN_ERR_STATE; }
    if (!state) { err = "NULL buffer"; return PN_ERR_INVALID; }
    PN_CUDA(cudaMemsetAsync(stage_d, 0, sizeof(double) * (size_t)L.n_state, stream));
    for (int c = 0; c < 8; ++c) {
      if (!L.active[c] || L.nm[c] == 0) continue;
      const long long n = L.npts[c] * L.nm[c];
      pack_points_kernel<T><<<grid_for(n), 256, 0, stream>>>(sstate + L.dev_off[c], stage_d + L.off_state[c],
                                                             L.shape[c][0], L.shape[c][1], L.shape[c][2], L.px[c],
                                                             L.nm[c], L.ms[c], 1.0 / scale_g, 1, class_bit(c, 0),
                                                             class_bit(c, 1), class_bit(c, 2), L.act[0], L.act[1],
                                                             L.act[2], nullptr);
      PN_CUDA(cudaGetLastError());
    }
    PN_CUDA(cudaMemcpyAsync(state, stage_d, sizeof(double) * (size_t)L.n_state, cudaMemcpyDeviceToHost, stream));
    PN_CUDA(cudaStreamSynchronize(stream));
    return PN_OK;
  }
};

}  // namespace pn
