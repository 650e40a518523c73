// pn_noalloc.cuh -- forward intensity march that takes all of its device scratch from a buffer
// the caller of this function provides (the library's static scratch array, see pn_noalloc.cu).
// It launches the same kernels as the handle-based path, directly on the caller's stream: no
// device allocation, no CUDA graph, no stream creation.
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "pn_solver.cuh"

namespace pn {

constexpr int NOALLOC_MAX_FACES = 1 << 16;

// host staging of the face lists; guarded because it is a single static buffer
inline std::mutex& noalloc_face_mutex() {
  static std::mutex m;
  return m;
}
inline int* noalloc_face_buffer() {
  static int buf[NOALLOC_MAX_FACES];
  return buf;
}

struct NoallocSegs {
  Seg seg[2][MAXSEG];
  int nseg[2];
  int nblk[2];
};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

template <int N>
int noalloc_forward(const pn_desc* d, unsigned char* scratch, size_t cap, const double* rho, const double* noa,
                    const double* acs, double* intensities, cudaStream_t s, std::string& err) {
  Layout L;
  int rc = L.init(d, err);
  if (rc) return rc;
  if (d->precision != PN_FP64) { err = "the no-allocation entry point runs the FP64 path only"; return PN_ERR_UNSUPPORTED; }
  if (L.nr < 1) { err = "the no-allocation entry point needs at least one x-ray line"; return PN_ERR_UNSUPPORTED; }
  if (!rho || !noa || !acs || !intensities) { err = "NULL buffer"; return PN_ERR_INVALID; }
  if ((rc = validate_desc(d, L, false, err))) return rc;
  const int ns = L.ns, ne = L.ne, nr = L.nr, N1 = N + 1;
  // advection table (compiled sparsity, values / h), checked as the handle path checks it
  double tab[Ord<N>::n_tab > 0 ? Ord<N>::n_tab : 1];
  if ((rc = advection_table<N>(d, L, tab, err))) return rc;

  std::lock_guard<std::mutex> lock(noalloc_face_mutex());
  int* faces_h = noalloc_face_buffer();
  NoallocSegs S;
  std::memset(&S, 0, sizeof(S));
  int nfaces = 0;
  struct Box { int cls; int lo[3], ext[3]; int f0, nf; };
  Box boxes[8];
  int nbox = 0;
  for (int c = 0; c < 8; ++c) {
    if (!L.active[c]) continue;
    Box b{};
    b.cls = c;
    int ilo[3], ihi[3];
    for (int k = 0; k < 3; ++k) {
      const int n = L.shape[c][k];
      if (!L.act[k]) { ilo[k] = 0; ihi[k] = 1; b.lo[k] = 0; b.ext[k] = 1; }
      else if (class_bit(c, k)) { ilo[k] = 1; ihi[k] = n - 1; b.lo[k] = 1; b.ext[k] = n - 2; }
      else { ilo[k] = 0; ihi[k] = n; b.lo[k] = 1; b.ext[k] = n - 2; }
      if (b.ext[k] < 0) b.ext[k] = 0;
    }
    b.f0 = nfaces;
    for (int kz = ilo[2]; kz < ihi[2]; ++kz)
      for (int jy = ilo[1]; jy < ihi[1]; ++jy)
        for (int ix = ilo[0]; ix < ihi[0]; ++ix) {
          const int cc[3] = {ix, jy, kz};
          bool face = false;
          for (int k = 0; k < 3; ++k)
            if (L.act[k] && !class_bit(c, k) && (cc[k] == 0 || cc[k] == L.shape[c][k] - 1)) face = true;
          if (!face) continue;
          if (nfaces >= NOALLOC_MAX_FACES) { err = "too many boundary cells for the no-allocation entry point"; return PN_ERR_NO_MEMORY; }
          faces_h[nfaces++] = pack_cell(ix, jy, kz);
        }
    b.nf = nfaces - b.f0;
    boxes[nbox++] = b;
  }

  // carve the scratch
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off = align256(off + bytes); return o; };
  const long long ncell = L.n_eee_cells;
  const size_t o_state = take(sizeof(double) * (size_t)L.slot_elems);
  const size_t o_rho = take(sizeof(double) * (size_t)L.rho_elems);
  const size_t o_wint = take(sizeof(double) * (size_t)(ncell * nr));
  const size_t o_bnd = take(sizeof(double) * (size_t)L.n_bnd);
  const size_t o_beam = take(sizeof(double) * (size_t)(L.n_beam > 0 ? L.n_beam : 1));
  const size_t o_xel = take(sizeof(int) * (size_t)nr);
  const size_t o_faces = take(sizeof(int) * (size_t)(nfaces > 0 ? nfaces : 1));
  const size_t o_sigma = take(sizeof(double) * (size_t)(ns + 1) * nr);
  const size_t o_weight = take(sizeof(double) * (size_t)(ns + 1));
  const size_t o_integral = take(sizeof(double) * (size_t)(ns + 1) * nr);
  // segments need the faces pointer: build them now
  int* faces_d = (int*)(scratch + o_faces);
  for (int q = 0; q < nbox; ++q) {
    const Box& b = boxes[q];
    const int par = class_parity(b.cls);
    if (b.ext[0] > 0 && b.ext[1] > 0 && b.ext[2] > 0) {
      Seg& g = S.seg[par][S.nseg[par]++];
      g.cls = b.cls;
      g.kind = 0;
      g.block0 = S.nblk[par];
      for (int k = 0; k < 3; ++k) { g.lo[k] = b.lo[k]; g.ext[k] = b.ext[k]; }
      g.tile_x = (b.ext[1] > 1 || b.ext[2] > 1) ? 32 : PBLOCK;
      g.tiles_x = (b.ext[0] + g.tile_x - 1) / g.tile_x;
      g.tiles_y = (b.ext[1] + PBLOCK / g.tile_x - 1) / (PBLOCK / g.tile_x);
      g.nblocks = g.tiles_x * g.tiles_y * b.ext[2];
      S.nblk[par] += g.nblocks;
    }
    if (b.nf > 0) {
      Seg& g = S.seg[par][S.nseg[par]++];
      g.cls = b.cls;
      g.kind = 1;
      g.block0 = S.nblk[par];
      g.tile_x = PBLOCK;
      g.tiles_x = g.tiles_y = 1;
      g.n_face = b.nf;
      g.faces = faces_d + b.f0;
      g.nblocks = (b.nf + PBLOCK - 1) / PBLOCK;
      S.nblk[par] += g.nblocks;
    }
  }
  if (S.nblk[0] == 0 || S.nblk[1] == 0) { err = "grid too small: a parity has no cells"; return PN_ERR_INVALID; }
  const size_t o_partial = take(sizeof(double) * (size_t)(ns + 1) * S.nblk[0] * nr);
  if (off > cap) {
    err = "problem needs " + std::to_string(off) + " bytes of scratch; the no-allocation entry point has " +
          std::to_string(cap);
    return PN_ERR_NO_MEMORY;
  }
  double* state = (double*)(scratch + o_state);
  double* rho_d = (double*)(scratch + o_rho);
  double* wint = (double*)(scratch + o_wint);
  double* bnd = (double*)(scratch + o_bnd);
  double* beam = (double*)(scratch + o_beam);
  int* xel = (int*)(scratch + o_xel);
  double* sigma = (double*)(scratch + o_sigma);
  double* weight = (double*)(scratch + o_weight);
  double* integral = (double*)(scratch + o_integral);
  double* partial = (double*)(scratch + o_partial);

  // the array keeps the previous call's contents: copy every table, zero what starts at zero
  PN_CUDA(cudaMemcpyAsync(bnd, d->boundary_fwd, sizeof(double) * (size_t)L.n_bnd, cudaMemcpyHostToDevice, s));
  if (L.n_beam) PN_CUDA(cudaMemcpyAsync(beam, d->beam_face, sizeof(double) * (size_t)L.n_beam, cudaMemcpyHostToDevice, s));
  PN_CUDA(cudaMemcpyAsync(xel, d->xray_element, sizeof(int) * (size_t)nr, cudaMemcpyHostToDevice, s));
  if (nfaces) PN_CUDA(cudaMemcpyAsync(faces_d, faces_h, sizeof(int) * (size_t)nfaces, cudaMemcpyHostToDevice, s));
  PN_CUDA(cudaMemcpyAsync(sigma, d->fwd_sigma, sizeof(double) * (size_t)(ns + 1) * nr, cudaMemcpyHostToDevice, s));
  PN_CUDA(cudaMemcpyAsync(weight, d->fwd_weight, sizeof(double) * (size_t)(ns + 1), cudaMemcpyHostToDevice, s));
  PN_CUDA(cudaMemsetAsync(state, 0, sizeof(double) * (size_t)L.slot_elems, s));
  PN_CUDA(cudaMemsetAsync(rho_d, 0, sizeof(double) * (size_t)L.rho_elems, s));
  PN_CUDA(cudaMemsetAsync(integral, 0, sizeof(double) * (size_t)(ns + 1) * nr, s));
  for (int c = 0; c < 8; ++c) {
    if (!L.active[c]) continue;
    const long long n = L.npts[c] * ne;
    unpack_points_kernel<double><<<grid_for(n), 256, 0, s>>>(rho + L.off_rho[c], rho_d + L.rho_off[c], L.shape[c][0],
                                                            L.shape[c][1], L.shape[c][2], L.px[c], ne, L.ms[c], 1.0);
    PN_CUDA(cudaGetLastError());
  }
  wint_kernel<<<grid_for(ncell * nr), 256, 0, s>>>(acs, noa, xel, wint, ncell, nr, ne);
  PN_CUDA(cudaGetLastError());

  // boundary block and beam pointers per class
  const double* bmat[3][8] = {{nullptr}};
  {
    long long o = 0;
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 8; ++c)
        if (class_bit(c, k)) {
          bmat[k][c] = bnd + o;
          o += (long long)L.nm[c] * L.nm[class_switch(c, k)];
        }
  }
  SubArgs<double, N> a;
  std::memset(&a, 0, sizeof(a));
  for (int c = 0; c < 8; ++c) {
    if (!L.active[c]) continue;
    for (int k = 0; k < 3; ++k) a.g[c].n[k] = L.shape[c][k];
    a.g[c].px = L.px[c];
    a.g[c].nm = L.nm[c];
    a.g[c].ms = L.ms[c];
    a.rd[c] = state + L.dev_off[c];
    a.wr[c] = state + L.dev_off[c];
    a.rho[c] = rho_d + L.rho_off[c];
    for (int k = 0; k < 3; ++k) a.bmat[k][c] = bmat[k][c];
    a.beam[c] = class_bit(c, 0) ? beam + L.beam_off[c] : nullptr;
  }
  for (int k = 0; k < 3; ++k) a.act[k] = L.act[k];
  a.ne = ne;
  a.nr = nr;
  a.scale_g = 1.0;
  a.acs = acs;
  a.noa = noa;
  a.wint = wint;
  for (int r = 0; r < nr; ++r) a.xel[r] = d->xray_element[r];
  for (int q = 0; q < Ord<N>::n_tab; ++q) a.tab[q] = tab[q];
  for (int i = 1; i <= ns; ++i) {
    for (int e = 0; e < ne; ++e) {
      a.s[e] = d->fwd_s[(long long)(i - 1) * ne + e];
      for (int l = 0; l <= N; ++l) a.c[e][l] = d->fwd_c[((long long)(i - 1) * ne + e) * N1 + l];
    }
    a.bc = d->fwd_bc[i - 1];
    for (int sub = 0; sub < 3; ++sub) {
      const int par = sub == 1 ? 0 : 1;
      a.dt = sub == 1 ? d->delta_e : d->delta_e / 2;
      a.nseg = S.nseg[par];
      for (int q = 0; q < a.nseg; ++q) a.seg[q] = S.seg[par][q];
      a.partial = sub == 1 ? partial + (long long)i * S.nblk[0] * nr : nullptr;
      substep_kernel<double, N, false><<<S.nblk[par], PBLOCK, 0, s>>>(a);
      PN_CUDA(cudaGetLastError());
    }
  }
  reduce_partials_kernel<<<ns, 256, 0, s>>>(partial, integral, S.nblk[0], nr, 1);
  PN_CUDA(cudaGetLastError());
  final_intensity_kernel<<<1, 32, 0, s>>>(integral, sigma, weight, intensities, ns + 1, nr, d->delta_e, d->dvol, 1.0);
  PN_CUDA(cudaGetLastError());
  if (d->flags & PN_FLAG_CHECK_FINITE) {
    double hI[MAXR];
    PN_CUDA(cudaStreamSynchronize(s));
    PN_CUDA(cudaMemcpy(hI, intensities, sizeof(double) * (size_t)nr, cudaMemcpyDeviceToHost));
    for (int r = 0; r < nr; ++r)
      if (!std::isfinite(hI[r])) { err = "intensities are not finite: the march diverged"; return PN_ERR_DIVERGED; }
  }
  // the face staging buffer was copied by a pageable-memory copy, which has completed on return
  return PN_OK;
}

}  // namespace pn
