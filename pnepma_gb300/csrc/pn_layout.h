// pn_layout.h -- geometry of a solve: class grids, the caller-facing (reference) layouts and the
// device layouts.  Host-only, shared by the C ABI and the per-order solvers.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/pnepma.h"

namespace pn {

inline int n_eee(int N) {
  auto fd = [](int a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); };
  int v = fd(N + 2) * fd(N + 4) / 2;
  return v > 0 ? v : 0;
}

inline int class_bit(int c, int d) { return (c >> (2 - d)) & 1; }
inline int class_switch(int c, int d) { return c ^ (4 >> d); }
inline int class_parity(int c) { return (class_bit(c, 0) + class_bit(c, 1) + class_bit(c, 2)) & 1; }

struct Layout {
  int N = 0, ne = 0, nr = 0, ns = 0;
  int M[3] = {1, 1, 1};
  int act[3] = {0, 0, 0};
  int nm[8] = {0};
  int shape[8][3] = {{0}};
  bool active[8] = {false};
  // caller (reference) layouts
  long long npts[8] = {0};
  long long off_state[8] = {0};
  long long off_rho[8] = {0};
  long long n_state = 0, n_rho = 0, n_eee_cells = 0;
  long long n_adv = 0, n_bnd = 0, n_beam = 0;
  long long beam_off[8] = {0};
  // device layouts (active classes; x pitch px, moment stride ms)
  int px[8] = {0};
  long long ms[8] = {0};
  long long dev_off[8] = {0};     // class offset inside one state slot (elements)
  long long slot_elems = 0;
  long long rho_off[8] = {0};     // per-class offset of [e][z][y][x] arrays
  long long rho_elems = 0;

  int init(const pn_desc* d, std::string& err) {
    if (d == nullptr) { err = "descriptor is NULL"; return PN_ERR_INVALID; }
    if (d->abi_version != PN_ABI_VERSION) { err = "descriptor abi_version does not match PN_ABI_VERSION"; return PN_ERR_INVALID; }
    N = d->order; ne = d->n_elements; nr = d->n_xrays; ns = d->n_steps;
    if (N < 0 || N > 31) { err = "order out of range"; return PN_ERR_INVALID; }
    if (ne < 1) { err = "n_elements must be >= 1"; return PN_ERR_INVALID; }
    if (nr < 0) { err = "n_xrays must be >= 0"; return PN_ERR_INVALID; }
    if (ns < 1) { err = "n_steps must be >= 1"; return PN_ERR_INVALID; }
    for (int k = 0; k < 3; ++k) {
      M[k] = d->n_points[k];
      if (M[k] < 1 || M[k] > 2000) { err = "n_points must be in 1..2000"; return PN_ERR_INVALID; }
      act[k] = M[k] > 1;
      if (act[k] && !(d->h[k] > 0.0)) { err = "grid step must be positive on a non-singleton axis"; return PN_ERR_INVALID; }
    }
    if (!act[0] && !act[1] && !act[2]) { err = "at least one axis must have more than one point"; return PN_ERR_INVALID; }
    const int sizes[8] = {n_eee(N), n_eee(N - 1), n_eee(N - 1), n_eee(N - 2),
                          n_eee(N - 1), n_eee(N - 2), n_eee(N - 2), n_eee(N - 3)};
    long long so = 0, ro = 0, bo = 0;
    for (int c = 0; c < 8; ++c) {
      nm[c] = sizes[c];
      long long np = 1;
      bool a = nm[c] > 0;
      for (int k = 0; k < 3; ++k) {
        shape[c][k] = (M[k] == 1) ? 1 : (class_bit(c, k) ? M[k] + 1 : M[k]);
        np *= shape[c][k];
        if (class_bit(c, k) && M[k] == 1) a = false;  // odd along a singleton axis: never advanced
      }
      active[c] = a;
      npts[c] = np;
      off_state[c] = so;
      off_rho[c] = ro;
      so += np * nm[c];
      ro += np * ne;
      if (class_bit(c, 0)) {
        beam_off[c] = bo;
        bo += (long long)shape[c][1] * shape[c][2] * nm[c];
      }
    }
    n_state = so;
    n_rho = ro;
    n_beam = bo;
    n_eee_cells = npts[0];
    n_adv = 0;
    n_bnd = 0;
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 8; ++c) {
        long long b = (long long)nm[c] * nm[class_switch(c, k)];
        n_adv += b;
        if (class_bit(c, k)) n_bnd += b;
      }
    long long off = 0, roff = 0;
    for (int c = 0; c < 8; ++c) {
      if (!active[c]) { px[c] = 0; ms[c] = 0; continue; }
      px[c] = (shape[c][0] + 7) / 8 * 8;
      ms[c] = (long long)px[c] * shape[c][1] * shape[c][2];
      dev_off[c] = off;
      off += ((ms[c] * nm[c] + 63) / 64) * 64;
      rho_off[c] = roff;
      roff += ((ms[c] * ne + 63) / 64) * 64;
    }
    slot_elems = off;
    rho_elems = roff;
    return PN_OK;
  }
};

}  // namespace pn
