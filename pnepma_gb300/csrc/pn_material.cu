// pn_material.cu -- the material on the device: component densities on the eight class grids,
// number of atoms and absorption factors from the material parameters, and the parameter gradient
// from the adjoint's outputs (pn_material_create / _fields / _pullback / _destroy).
//
// Reference: pn_solver/pn_parametrizations/pn_material.jl (the four material models and their SC
// variants, with their hand-written pullbacks), pn_parametrization_const.jl,
// pn_parametrization_boxed.jl:137-175, pn_parametrization_bilinear.jl:122-130 with
// biliner_interp.jl:5-36,63-111,163-218 (point location, trilinear value and its pullback),
// pn_material_utils.jl:74-91 (all eight grids), x_ray_intensities.jl:43-153 (number of atoms,
// absorption factors and their pullbacks).
//
// This unit is compiled with -fmad=false: every product and sum below rounds as the reference's
// Julia code (which does not contract) rounds it, so the point location -- the floor of a
// quotient, which a fused multiply-add could move across a box boundary -- and the trilinear
// weights are the ones the reference computes from the same inputs.
//
// Work decomposition.  Fields: one thread per grid point (all classes in one launch); absorption:
// one warp per eee cell, its lanes over the ray's samples, the exponent reduced with shuffles.
// Pullbacks: the same decomposition; each contribution goes to one parameter vector (a box, a
// knot or the embedding), and lanes of a warp that hit the same vector add their contributions in
// shared memory before one FP64 atomic per component, so a coarse parametrisation (few boxes or
// knots, a constant) does not serialise on a handful of addresses.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pnepma.h"
#include "pn_trace.h"

namespace pn {
void set_last_error(const std::string& msg);  // pn_capi.cu
}

namespace {

constexpr int MAT_MAXE = 8;   // elements
constexpr int MAT_MAXR = 8;   // x-ray lines
constexpr int MAT_BLOCK = 256;
constexpr long long KEY_NONE = -1;

struct MatDev {
  int model, sc, par, ne, npar, nr, nint;
  int M[3];
  int shape[8][3];             // class grid (nx, ny, nz)
  long long off[9];            // first point of each class (prefix sums; off[8] = all points)
  long long n_eee;
  const double* coords[3][2];  // device: per axis, even and odd points
  int sl_n[3], sl_off[3];
  double sl_ref[3], sl_step[3];
  const double* sl_vals[3];    // device, vector form only
  int nb[3];                   // boxes (Boxed) or knots (Bilinear) per axis
  long long emb;               // index of the embedding parameter vector
  double rho_pure[MAT_MAXE], atom_mass[MAT_MAXE];
  double mac[MAT_MAXR][MAT_MAXE];
  double det[3], beam_x;
};

// ------------------------------------------------------------------ point location

// find_index_smaller_and_partition (biliner_interp.jl:5-36): 1-based index i and partition p
__device__ __forceinline__ void locate_axis(const MatDev& m, int d, double x, long long& i, double& p) {
  const int n = m.sl_n[d];
  if (n == 1) {   // the reference asserts that x is the single slice value
    i = 1;
    p = 0.0;
    return;
  }
  const double* v = m.sl_vals[d];
  if (!v) {       // StepRangeLen form
    const double ref = m.sl_ref[d], step = m.sl_step[d];
    const double dd = x - ref;
    const double f = floor(dd / step);
    i = (long long)f + m.sl_off[d];
    p = (dd - f * step) / step;
    return;
  }
  // Vector form: the reference walks i = 1, 2, ... while x > v[i+1] and i < n - 1, i.e. it stops
  // at the first i with x <= v[i+1] (or at n - 1); slices are increasing, so that is a binary
  // search for the first 0-based k >= 1 with x <= v[k], then i = k.
  int lo = 1, hi = n - 1;     // answer in [1, n-1]
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (x <= v[mid]) hi = mid;
    else lo = mid + 1;
  }
  long long ii = lo;          // 1-based i: the interval [v[ii-1], v[ii]] in 0-based values
  const double dd = (x - v[ii - 1]) / (v[ii] - v[ii - 1]);
  if (dd < 0.0) ii -= 1;
  else if (dd > 1.0) ii += 1;
  i = ii;
  p = dd;
}

__device__ __forceinline__ bool approx_zero(double a) { return fabs(a) < 1e-20; }

// Terms of the parametrisation at a point: parameter-vector indices (m.emb for the embedding)
// and weights, in the reference's summation order.  Returns the number of terms (1..8).
__device__ int param_terms(const MatDev& m, const double x[3], long long key[8], double w[8]) {
  if (m.par == PN_PAR_CONST) {
    key[0] = 0;
    w[0] = 1.0;
    return 1;
  }
  long long idx[3];
  double p[3];
  for (int d = 0; d < 3; ++d) locate_axis(m, d, x[d], idx[d], p[d]);
  if (m.par == PN_PAR_BOXED) {
    // pn_parametrization_boxed.jl:137-155
    bool inside = true;
    for (int d = 0; d < 3; ++d) {
      if (idx[d] == m.sl_n[d] && approx_zero(p[d])) idx[d] -= 1;
      inside = inside && idx[d] >= 1 && idx[d] <= m.sl_n[d] - 1;
    }
    key[0] = inside ? ((idx[2] - 1) * m.nb[1] + (idx[1] - 1)) * m.nb[0] + (idx[0] - 1) : m.emb;
    w[0] = 1.0;
    return 1;
  }
  // Bilinear (biliner_interp.jl:63-111).  The branch taken depends on which partitions are
  // (approximately) zero; its terms are the corners over the remaining axes, ordered by the
  // number of offset axes and then x before y before z, each weighted by the product over those
  // axes (x, y, z order) of p or 1 - p -- the order in which the reference writes them.
  int act = 0;
  for (int d = 0; d < 3; ++d)
    if (!approx_zero(p[d])) act |= 1 << d;
  const int order[8] = {0, 1, 2, 4, 3, 5, 6, 7};
  int n = 0;
  for (int t = 0; t < 8; ++t) {
    const int s = order[t];
    if (s & ~act) continue;
    double ww = 1.0;
    bool in = true;
    long long c[3];
    for (int d = 0; d < 3; ++d) {
      const int b = (s >> d) & 1;
      c[d] = idx[d] + b;
      if (act & (1 << d)) ww = ww * (b ? p[d] : 1.0 - p[d]);
      in = in && c[d] >= 1 && c[d] <= m.nb[d];
    }
    key[n] = in ? ((c[2] - 1) * m.nb[1] + (c[1] - 1)) * m.nb[0] + (c[0] - 1) : m.emb;
    w[n] = ww;
    ++n;
  }
  return n;
}

// parametrization! at a point: p[0..npar)
__device__ void param_value(const MatDev& m, const double* __restrict__ P, const double x[3], double* p) {
  long long key[8];
  double w[8];
  const int n = param_terms(m, x, key, w);
  if (n == 1) {
    for (int q = 0; q < m.npar; ++q) p[q] = P[key[0] * m.npar + q];
    return;
  }
  for (int q = 0; q < m.npar; ++q) {
    double s = w[0] * P[key[0] * m.npar + q];
    for (int t = 1; t < n; ++t) s = s + w[t] * P[key[t] * m.npar + q];
    p[q] = s;
  }
}

// full component vector (the SC variants append 1 - sum of the others)
__device__ __forceinline__ void full_vector(const MatDev& m, const double* p, double* f) {
  for (int q = 0; q < m.npar; ++q) f[q] = p[q];
  if (m.sc) {
    double s = 0.0;
    for (int q = 0; q < m.npar; ++q) s = s + p[q];
    f[m.ne - 1] = 1.0 - s;
  }
}

// component_densities! (pn_material.jl:71-73,114-123,172-181,233-244)
__device__ void densities_from(const MatDev& m, const double* p, double* rho) {
  double f[MAT_MAXE];
  full_vector(m, p, f);
  const int ne = m.ne;
  switch (m.model) {
    case PN_MAT_MASS_CONCENTRATION:
      for (int e = 0; e < ne; ++e) rho[e] = f[e];
      break;
    case PN_MAT_VOLUME_FRACTION:
      for (int e = 0; e < ne; ++e) rho[e] = f[e] * m.rho_pure[e];
      break;
    case PN_MAT_LINEAR_DENSITY: {
      double dt = 0.0;
      for (int e = 0; e < ne; ++e) dt = dt + f[e] * m.rho_pure[e];
      for (int e = 0; e < ne; ++e) rho[e] = f[e] * dt;
      break;
    }
    default: {  // PN_MAT_MASS_FRACTION
      double R = 0.0;
      for (int e = 0; e < ne; ++e) R = R + f[e] / m.rho_pure[e];
      for (int e = 0; e < ne; ++e) rho[e] = f[e] / R;
    }
  }
}

// component_densities_pullback! up to the parametrisation (pn_material.jl:75-77,125-134,183-197,
// 246-264): the parameter-space cotangent pb[0..npar) of rho_bar at a point with value p
__device__ void model_pullback(const MatDev& m, const double* p, const double* rb, double* pb) {
  const int ne = m.ne;
  double g[MAT_MAXE];
  switch (m.model) {
    case PN_MAT_MASS_CONCENTRATION:
      for (int e = 0; e < ne; ++e) g[e] = rb[e];
      break;
    case PN_MAT_VOLUME_FRACTION:
      for (int e = 0; e < ne; ++e) g[e] = rb[e] * m.rho_pure[e];
      break;
    case PN_MAT_LINEAR_DENSITY: {
      double f[MAT_MAXE];
      full_vector(m, p, f);
      double dpr = 0.0, dpb = 0.0;
      for (int e = 0; e < ne; ++e) dpr = dpr + f[e] * m.rho_pure[e];
      for (int e = 0; e < ne; ++e) dpb = dpb + f[e] * rb[e];
      for (int e = 0; e < ne; ++e) g[e] = rb[e] * dpr + m.rho_pure[e] * dpb;
      break;
    }
    default: {  // PN_MAT_MASS_FRACTION
      double f[MAT_MAXE];
      full_vector(m, p, f);
      double R = 0.0, d = 0.0;
      for (int e = 0; e < ne; ++e) R = R + f[e] / m.rho_pure[e];
      for (int e = 0; e < ne; ++e) d = d + f[e] * rb[e];
      const double Rb = -d / (R * R);
      for (int e = 0; e < ne; ++e) g[e] = rb[e] / R + Rb / m.rho_pure[e];
    }
  }
  if (m.sc)
    for (int q = 0; q < m.npar; ++q) pb[q] = g[q] - g[ne - 1];
  else
    for (int q = 0; q < m.npar; ++q) pb[q] = g[q];
}

__device__ __forceinline__ bool model_needs_value(const MatDev& m) {
  return m.model == PN_MAT_LINEAR_DENSITY || m.model == PN_MAT_MASS_FRACTION;
}

// Coordinates and class of global point q (all eight grids, classes concatenated, x fastest).
__device__ __forceinline__ int point_of(const MatDev& m, long long q, double x[3], long long& local) {
  int c = 0;
  while (c < 7 && q >= m.off[c + 1]) ++c;
  local = q - m.off[c];
  const int nx = m.shape[c][0], ny = m.shape[c][1];
  const long long i = local % nx, r = local / nx;
  const long long j = r % ny, k = r / ny;
  const long long ijk[3] = {i, j, k};
  for (int d = 0; d < 3; ++d) {
    const int odd = (c >> (2 - d)) & 1;
    x[d] = m.coords[d][odd][ijk[d]];
  }
  return c;
}

__device__ __forceinline__ void eee_point(const MatDev& m, long long cell, double x[3]) {
  const long long i = cell % m.M[0], r = cell / m.M[0];
  const long long j = r % m.M[1], k = r / m.M[1];
  x[0] = m.coords[0][0][i];
  x[1] = m.coords[1][0][j];
  x[2] = m.coords[2][0][k];
}

// ray of an eee cell (compute_absorption_coefficient!, x_ray_intensities.jl:100-113)
__device__ __forceinline__ void ray_of(const MatDev& m, const double o[3], double dir[3], double& lam, double& dx) {
  for (int d = 0; d < 3; ++d) dir[d] = m.det[d] - o[d];
  lam = fmax((m.beam_x - o[0]) / dir[0], 0.0);
  const double nrm = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
  dx = nrm * lam / m.nint;
}

// sample k of range(0, lam, length = nint) and its point
__device__ __forceinline__ void sample_point(const MatDev& m, const double o[3], const double dir[3], double lam, int k,
                                             double x[3]) {
  const double l = m.nint > 1 ? lam * ((double)k / (double)(m.nint - 1)) : 0.0;
  for (int d = 0; d < 3; ++d) x[d] = o[d] + l * dir[d];
}

// ------------------------------------------------------------------ kernels

__global__ void __launch_bounds__(MAT_BLOCK) mat_fields_kernel(const __grid_constant__ MatDev m,
                                                               const double* __restrict__ P, double* __restrict__ rho,
                                                               double* __restrict__ noa) {
  const long long n = m.off[8];
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    double x[3], p[MAT_MAXE], r[MAT_MAXE];
    long long local;
    const int c = point_of(m, q, x, local);
    param_value(m, P, x, p);
    densities_from(m, p, r);
    if (rho)
      for (int e = 0; e < m.ne; ++e) rho[q * m.ne + e] = r[e];
    if (noa && c == 0)
      for (int e = 0; e < m.ne; ++e) noa[local * m.ne + e] = r[e] / m.atom_mass[e];
  }
}

// one warp per eee cell
__global__ void __launch_bounds__(MAT_BLOCK) mat_absorption_kernel(const __grid_constant__ MatDev m,
                                                                   const double* __restrict__ P,
                                                                   double* __restrict__ acs) {
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long cell = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); cell < m.n_eee; cell += nw) {
    double o[3], dir[3], lam, dx;
    eee_point(m, cell, o);
    ray_of(m, o, dir, lam, dx);
    double acc[MAT_MAXR];
    for (int r = 0; r < m.nr; ++r) acc[r] = 0.0;
    for (int k = lane; k < m.nint; k += 32) {
      double x[3], p[MAT_MAXE], rho[MAT_MAXE];
      sample_point(m, o, dir, lam, k, x);
      param_value(m, P, x, p);
      densities_from(m, p, rho);
      for (int r = 0; r < m.nr; ++r) {
        double s = 0.0;
        for (int e = 0; e < m.ne; ++e) s = s + m.mac[r][e] * rho[e];
        acc[r] = acc[r] - s;
      }
    }
    for (int r = 0; r < m.nr; ++r) {
      double v = acc[r];
      for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o2);
      acc[r] = v;
    }
    if (lane == 0)
      for (int r = 0; r < m.nr; ++r) acs[cell * m.nr + r] = exp(acc[r] * dx);
  }
}

// Add vals[0..npar) (per lane) into G[key * npar ..]; lanes with the same key combine first.  Every
// lane of the warp calls this with the same npar; key < 0 contributes nothing.
__device__ __forceinline__ void warp_scatter(double* __restrict__ G, long long key, const double* vals, int npar,
                                             double* sm /* [MAT_MAXE][32] of this warp */) {
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(0xffffffffu, (unsigned long long)key);
  for (int q = 0; q < npar; ++q) sm[q * 32 + lane] = vals[q];
  __syncwarp();
  if (key >= 0 && lane == __ffs(peers) - 1) {
    for (int q = 0; q < npar; ++q) {
      double s = 0.0;
      for (unsigned b = peers; b; b &= b - 1) s += sm[q * 32 + (__ffs(b) - 1)];
      atomicAdd(G + key * npar + q, s);
    }
  }
  __syncwarp();
}

// Scatter the cotangent pb of the parametrisation value at x (parametrization_pullback!): every
// term gets weight * pb.  Called by all lanes; `live` false contributes nothing.
__device__ __forceinline__ void scatter_point(const MatDev& m, double* __restrict__ G, bool live, const double x[3],
                                              const double* pb, double* sm) {
  long long key[8];
  double w[8];
  int n = 0;
  if (live) n = param_terms(m, x, key, w);
  const int nmax = m.par == PN_PAR_BILINEAR ? 8 : 1;
  for (int t = 0; t < nmax; ++t) {
    double v[MAT_MAXE];
    long long k = KEY_NONE;
    if (t < n) {
      k = key[t];
      if (n == 1)
        for (int q = 0; q < m.npar; ++q) v[q] = pb[q];
      else
        for (int q = 0; q < m.npar; ++q) v[q] = w[t] * pb[q];
    } else {
      for (int q = 0; q < m.npar; ++q) v[q] = 0.0;
    }
    warp_scatter(G, k, v, m.npar, sm);
  }
}

// component_densities_pullback on all eight grids and compute_number_of_atoms_pullback on the eee
// grid; one thread per point, every lane of a warp through the same iterations
__global__ void __launch_bounds__(MAT_BLOCK) mat_pullback_grid_kernel(const __grid_constant__ MatDev m,
                                                                      const double* __restrict__ P,
                                                                      const double* __restrict__ rho_bar,
                                                                      const double* __restrict__ noa_bar,
                                                                      double* __restrict__ G) {
  __shared__ double smem[MAT_BLOCK / 32][MAT_MAXE * 32];
  double* sm = smem[threadIdx.x >> 5];
  const long long n = m.off[8];
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (blockIdx.x * (long long)blockDim.x + threadIdx.x) & ~31LL; base < n; base += stride) {
    const long long q = base + (threadIdx.x & 31);
    const bool valid = q < n;
    double x[3] = {0.0, 0.0, 0.0}, p[MAT_MAXE], pb[MAT_MAXE];
    long long local = 0;
    int c = -1;
    if (valid) c = point_of(m, q, x, local);
    for (int pass = 0; pass < 2; ++pass) {
      // pass 0: rho_bar at this point (every grid); pass 1: noa_bar / atom_mass (eee points)
      double rb[MAT_MAXE];
      bool live = false;
      if (valid && pass == 0 && rho_bar) {
        for (int e = 0; e < m.ne; ++e) {
          rb[e] = rho_bar[q * m.ne + e];
          live = live || rb[e] != 0.0;
        }
      } else if (valid && pass == 1 && noa_bar && c == 0) {
        for (int e = 0; e < m.ne; ++e) {
          rb[e] = noa_bar[local * m.ne + e] / m.atom_mass[e];
          live = live || rb[e] != 0.0;
        }
      }
      if (live) {
        if (model_needs_value(m)) param_value(m, P, x, p);
        model_pullback(m, p, rb, pb);
      }
      if (__any_sync(0xffffffffu, live)) scatter_point(m, G, live, x, pb, sm);
    }
  }
}

// compute_absorption_coefficient_pullback (x_ray_intensities.jl:131-153): one warp per eee cell
__global__ void __launch_bounds__(MAT_BLOCK) mat_pullback_absorption_kernel(const __grid_constant__ MatDev m,
                                                                            const double* __restrict__ P,
                                                                            const double* __restrict__ acs,
                                                                            const double* __restrict__ acs_bar,
                                                                            double* __restrict__ G) {
  __shared__ double smem[MAT_BLOCK / 32][MAT_MAXE * 32];
  double* sm = smem[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long cell = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); cell < m.n_eee; cell += nw) {
    double o[3], dir[3], lam, dx;
    eee_point(m, cell, o);
    ray_of(m, o, dir, lam, dx);
    // acs_adj = -acs .* dx .* acs_bar;  rho_adj = macs * acs_adj  (the same at every sample)
    double aa[MAT_MAXR], radj[MAT_MAXE];
    bool any = false;
    for (int r = 0; r < m.nr; ++r) {
      aa[r] = -acs[cell * m.nr + r] * dx * acs_bar[cell * m.nr + r];
      any = any || aa[r] != 0.0;
    }
    if (!any) continue;   // warp-uniform: every lane of the warp handles this cell
    for (int e = 0; e < m.ne; ++e) {
      double s = 0.0;
      for (int r = 0; r < m.nr; ++r) s = s + m.mac[r][e] * aa[r];
      radj[e] = s;
    }
    double pb_const[MAT_MAXE];
    const bool need_p = model_needs_value(m);
    if (!need_p) model_pullback(m, nullptr, radj, pb_const);
    for (int k0 = 0; k0 < m.nint; k0 += 32) {
      const int k = k0 + lane;
      const bool live = k < m.nint;
      double x[3] = {0.0, 0.0, 0.0}, p[MAT_MAXE], pb[MAT_MAXE];
      if (live) {
        sample_point(m, o, dir, lam, k, x);
        if (need_p) {
          param_value(m, P, x, p);
          model_pullback(m, p, radj, pb);
        } else {
          for (int q = 0; q < m.npar; ++q) pb[q] = pb_const[q];
        }
      }
      scatter_point(m, G, live, x, pb, sm);
    }
  }
}

int grid_for(long long work, int per_block) {
  long long b = (work + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > 152LL * 16) b = 152LL * 16;
  return (int)b;
}

}  // namespace

struct pn_material {
  MatDev dev;
  int device = -1;
  int64_t n_params = 0;
  std::vector<void*> allocs;
  std::string err;
};

namespace {

int fail(pn_material* m, int code, const std::string& msg) {
  if (m) m->err = msg;
  pn::set_last_error(msg);
  return code;
}

bool valid_slices(const pn_slices& s, std::string& why) {
  if (s.n < 1) {
    why = "slices need at least one value";
    return false;
  }
  if (s.values) {
    for (int i = 0; i + 1 < s.n; ++i)
      if (!(s.values[i] < s.values[i + 1])) {
        why = "vector slices must be strictly increasing";
        return false;
      }
  } else if (s.n > 1 && !(std::isfinite(s.step) && s.step != 0.0 && std::isfinite(s.ref))) {
    why = "range slices need a finite non-zero step and a finite reference value";
    return false;
  }
  return true;
}

}  // namespace

extern "C" {

int pn_material_create(const pn_material_desc* d, pn_material** out, int64_t* n_params) {
  if (!d || !out) return fail(nullptr, PN_ERR_INVALID, "descriptor or output pointer is NULL");
  *out = nullptr;
  if (d->model < PN_MAT_MASS_CONCENTRATION || d->model > PN_MAT_MASS_FRACTION)
    return fail(nullptr, PN_ERR_INVALID, "unknown material model");
  if (d->parametrization < PN_PAR_CONST || d->parametrization > PN_PAR_BILINEAR)
    return fail(nullptr, PN_ERR_INVALID, "unknown parametrisation");
  if (d->n_elements < 1 || d->n_elements > MAT_MAXE)
    return fail(nullptr, PN_ERR_UNSUPPORTED, "material with 1 to 8 elements only");
  if (d->sc && (d->model == PN_MAT_MASS_CONCENTRATION || d->n_elements < 2))
    return fail(nullptr, PN_ERR_INVALID, "an SC variant needs a volume-fraction, linear-density or mass-fraction "
                                         "model and at least two elements");
  if (d->n_xrays < 0 || d->n_xrays > MAT_MAXR) return fail(nullptr, PN_ERR_UNSUPPORTED, "0 to 8 x-ray lines only");
  if (d->n_xrays > 0 && (d->n_int_points < 1 || !d->mac))
    return fail(nullptr, PN_ERR_INVALID, "absorption factors need n_int_points >= 1 and the mac table");
  if (!d->coords) return fail(nullptr, PN_ERR_INVALID, "coords is NULL");
  if (d->model != PN_MAT_MASS_CONCENTRATION && !d->rho_pure) return fail(nullptr, PN_ERR_INVALID, "rho_pure is NULL");
  for (int k = 0; k < 3; ++k)
    if (d->n_points[k] < 1) return fail(nullptr, PN_ERR_INVALID, "n_points must be >= 1");
  if (d->parametrization == PN_PAR_BILINEAR)
    for (int k = 0; k < 3; ++k)
      if (d->slices[k].values) return fail(nullptr, PN_ERR_INVALID, "bilinear knots must be in range form");
  if (d->parametrization != PN_PAR_CONST)
    for (int k = 0; k < 3; ++k) {
      std::string why;
      if (!valid_slices(d->slices[k], why)) return fail(nullptr, PN_ERR_INVALID, why);
    }

  pn_material* m = new pn_material;
  MatDev& g = m->dev;
  std::memset(&g, 0, sizeof(g));
  g.model = d->model;
  g.sc = d->sc ? 1 : 0;
  g.par = d->parametrization;
  g.ne = d->n_elements;
  g.npar = g.sc ? g.ne - 1 : g.ne;
  g.nr = d->n_xrays;
  g.nint = d->n_xrays > 0 ? d->n_int_points : 0;
  long long n_vec = 1;
  for (int k = 0; k < 3; ++k) {
    g.M[k] = d->n_points[k];
    if (g.par != PN_PAR_CONST) {
      g.sl_n[k] = d->slices[k].n;
      g.sl_off[k] = d->slices[k].offset;
      g.sl_ref[k] = d->slices[k].ref;
      g.sl_step[k] = d->slices[k].step;
      g.nb[k] = g.par == PN_PAR_BOXED ? d->slices[k].n - 1 : d->slices[k].n;
      n_vec *= g.nb[k];
    }
  }
  g.emb = g.par == PN_PAR_CONST ? 0 : n_vec;
  m->n_params = g.par == PN_PAR_CONST ? (int64_t)g.npar : (int64_t)(n_vec + 1) * g.npar;
  long long tot = 0;
  for (int c = 0; c < 8; ++c) {
    g.off[c] = tot;
    long long np = 1;
    for (int k = 0; k < 3; ++k) {
      const int odd = (c >> (2 - k)) & 1;
      g.shape[c][k] = g.M[k] == 1 ? 1 : g.M[k] + odd;
      np *= g.shape[c][k];
    }
    tot += np;
  }
  g.off[8] = tot;
  g.n_eee = (long long)g.M[0] * g.M[1] * g.M[2];
  for (int e = 0; e < g.ne; ++e) {
    g.rho_pure[e] = d->rho_pure ? d->rho_pure[e] : 0.0;
    g.atom_mass[e] = d->atom_mass ? d->atom_mass[e] : 1.0;
  }
  for (int r = 0; r < g.nr; ++r)
    for (int e = 0; e < g.ne; ++e) g.mac[r][e] = d->mac[r * g.ne + e];
  for (int k = 0; k < 3; ++k) g.det[k] = d->detector[k];
  g.beam_x = d->beam_x;

  // device tables: coordinates (even then odd per axis) and vector slices
  if (cudaGetDevice(&m->device) != cudaSuccess) {
    cudaGetLastError();
    delete m;
    return fail(nullptr, PN_ERR_NO_DEVICE, "no CUDA device is available");
  }
  size_t ncoord = 0;
  for (int k = 0; k < 3; ++k) ncoord += (size_t)g.M[k] + (g.M[k] == 1 ? 1 : g.M[k] + 1);
  size_t nsl = 0;
  for (int k = 0; k < 3; ++k)
    if (g.par == PN_PAR_BOXED && d->slices[k].values) nsl += (size_t)d->slices[k].n;
  double* dbuf = nullptr;
  if (cudaMalloc(&dbuf, sizeof(double) * (ncoord + nsl)) != cudaSuccess) {
    cudaGetLastError();
    delete m;
    return fail(nullptr, PN_ERR_NO_MEMORY, "cudaMalloc of the material tables failed");
  }
  m->allocs.push_back(dbuf);
  std::vector<double> host(ncoord + nsl);
  size_t at = 0;
  for (int k = 0; k < 3; ++k) {
    const size_t ne_ = (size_t)g.M[k], no_ = g.M[k] == 1 ? 1 : (size_t)g.M[k] + 1;
    std::memcpy(host.data() + at, d->coords + at, sizeof(double) * (ne_ + no_));
    g.coords[k][0] = dbuf + at;
    g.coords[k][1] = dbuf + at + ne_;
    at += ne_ + no_;
  }
  for (int k = 0; k < 3; ++k) {
    g.sl_vals[k] = nullptr;
    if (g.par == PN_PAR_BOXED && d->slices[k].values) {
      std::memcpy(host.data() + at, d->slices[k].values, sizeof(double) * d->slices[k].n);
      g.sl_vals[k] = dbuf + at;
      at += d->slices[k].n;
    }
  }
  if (cudaMemcpy(dbuf, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    pn_material_destroy(m);
    return fail(nullptr, PN_ERR_CUDA, "copy of the material tables failed");
  }
  if (n_params) *n_params = m->n_params;
  *out = m;
  return PN_OK;
}

int pn_material_fields(pn_material* m, const double* params, double* rho, double* noa, double* acs, void* stream) {
  if (!m || !params) return fail(m, PN_ERR_INVALID, "material handle or params is NULL");
  pn::TraceRange trace("pn_material_fields");
  const MatDev& g = m->dev;
  cudaStream_t s = (cudaStream_t)stream;
  if (rho || noa) mat_fields_kernel<<<grid_for(g.off[8], MAT_BLOCK), MAT_BLOCK, 0, s>>>(g, params, rho, noa);
  if (acs && g.nr > 0)
    mat_absorption_kernel<<<grid_for(g.n_eee, MAT_BLOCK / 32), MAT_BLOCK, 0, s>>>(g, params, acs);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(m, PN_ERR_CUDA, std::string("material kernels: ") + cudaGetErrorString(e));
  return PN_OK;
}

int pn_material_pullback(pn_material* m, const double* params, const double* rho_bar, const double* noa_bar,
                         const double* acs, const double* acs_bar, double* params_bar, void* stream) {
  if (!m || !params || !params_bar) return fail(m, PN_ERR_INVALID, "material handle, params or params_bar is NULL");
  if (acs_bar && !acs) return fail(m, PN_ERR_INVALID, "acs_bar needs the forward's acs");
  pn::TraceRange trace("pn_material_pullback");
  const MatDev& g = m->dev;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(params_bar, 0, sizeof(double) * (size_t)m->n_params, s) != cudaSuccess) {
    cudaGetLastError();
    return fail(m, PN_ERR_CUDA, "clearing params_bar failed");
  }
  if (rho_bar || noa_bar)
    mat_pullback_grid_kernel<<<grid_for(g.off[8], MAT_BLOCK), MAT_BLOCK, 0, s>>>(g, params, rho_bar, noa_bar,
                                                                                 params_bar);
  if (acs_bar && g.nr > 0)
    mat_pullback_absorption_kernel<<<grid_for(g.n_eee, MAT_BLOCK / 32), MAT_BLOCK, 0, s>>>(g, params, acs, acs_bar,
                                                                                            params_bar);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(m, PN_ERR_CUDA, std::string("material pullback kernels: ") + cudaGetErrorString(e));
  return PN_OK;
}

void pn_material_destroy(pn_material* m) {
  if (!m) return;
  for (void* p : m->allocs) cudaFree(p);
  delete m;
}

}  // extern "C"
