// pn_util.cuh -- layout conversion and reduction kernels (reference layout <-> device layout).
#pragma once

#include <cuda_runtime.h>

namespace pn {

// caller layout [point][v] of one class -> device [v][z][y][x] (pitched), times `mul`, converted to T
template <class T>
static __global__ void unpack_points_kernel(const double* __restrict__ src, T* __restrict__ dst, int nx, int ny, int nz,
                                     int px, int nv, long long ms, double mul) {
  const long long np = (long long)nx * ny * nz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < np * nv;
       q += (long long)gridDim.x * blockDim.x) {
    const long long p = q / nv;
    const int v = (int)(q - p * nv);
    const int i = (int)(p % nx);
    const long long r = p / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    dst[v * ms + ((long long)k * ny + j) * px + i] = T(src[q] * mul);
  }
}

// device [v][z][y][x] -> caller [point][v], times `mul`
template <class T>
static __global__ void pack_points_kernel(const T* __restrict__ src, double* __restrict__ dst, int nx, int ny, int nz,
                                   int px, int nv, long long ms, double mul, int zero_multi_ghost,
                                   int ox, int oy, int oz, int ax, int ay, int az, const double* __restrict__ mulp) {
  if (mulp) mul *= mulp[0];
  const long long np = (long long)nx * ny * nz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < np * nv;
       q += (long long)gridDim.x * blockDim.x) {
    const long long p = q / nv;
    const int v = (int)(q - p * nv);
    const int i = (int)(p % nx);
    const long long r = p / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    double val = double(src[v * ms + ((long long)k * ny + j) * px + i]) * mul;
    if (zero_multi_ghost) {
      const int gx = ox && ax && (i == 0 || i == nx - 1);
      const int gy = oy && ay && (j == 0 || j == ny - 1);
      const int gz = oz && az && (k == 0 || k == nz - 1);
      if (gx + gy + gz >= 2) val = 0.0;
    }
    dst[q] = val;
  }
}

// W[cell][r] = ACS[cell][r] * NOA[cell][el_r]
static __global__ void wint_kernel(const double* __restrict__ acs, const double* __restrict__ noa,
                            const int* __restrict__ xel, double* __restrict__ w, long long ncell, int nr,
                            int ne) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < ncell * nr;
       q += (long long)gridDim.x * blockDim.x) {
    const long long c = q / nr;
    const int r = (int)(q - c * nr);
    w[q] = acs[q] * noa[c * ne + xel[r]];
  }
}

// integral[s][r] = sum over blocks of partial[s][b][r], in block order (one block per step)
static __global__ void reduce_partials_kernel(const double* __restrict__ partial, double* __restrict__ integral,
                                       int nblk, int nr, int first_step) {
  const int s = blockIdx.x + first_step;
  __shared__ double buf[256];
  for (int r = 0; r < nr; ++r) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += partial[((long long)s * nblk + b) * nr + r];
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) buf[threadIdx.x] += buf[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) integral[(long long)s * nr + r] = buf[0];
    __syncthreads();
  }
}

// field[cell][r] += u_eee0[cell] * dE * sigma_r * w   (integrate_step_and_add_x_ray_generation!)
template <class T>
static __global__ void generation_kernel(const T* __restrict__ u0, double* __restrict__ field, int nx, int ny, int nz,
                                  int px, int nr, double dE, const double* __restrict__ sigma, double w,
                                  double mul) {
  const long long np = (long long)nx * ny * nz;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np;
       p += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(p % nx);
    const long long r = p / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    const double u = double(u0[((long long)k * ny + j) * px + i]) * mul;
    for (int q = 0; q < nr; ++q) field[p * nr + q] = field[p * nr + q] + u * dE * sigma[q] * w;
  }
}

// scale a double buffer in place by mul * (*mulp)
static __global__ void scale_kernel(double* __restrict__ x, long long n, double mul, const double* __restrict__ mulp) {
  const double f = mulp ? mul * mulp[0] : mul;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    x[q] *= f;
}

// Copy the cotangent to the device buffer the adjoint graph reads, scaled by a power of two that
// keeps the FP32 adjoint source near unity (FP64: no scaling), and store the factor that undoes
// the scaling of the outputs: out_mul[0] = 1 / (scale_g * scale_i).
static __global__ void prep_ibar_kernel(const double* __restrict__ ibar_in, double* __restrict__ ibar_d,
                                        double* __restrict__ out_mul, int nr, double src_mag, int fp32,
                                        double scale_g) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double m = 0.0;
  for (int r = 0; r < nr; ++r) m = fmax(m, fabs(ibar_in[r]));
  double sc = 1.0;
  const double q = m * src_mag;
  if (fp32 && q > 0.0 && isfinite(q)) sc = ldexp(1.0, -(int)llrint(log2(q)));
  for (int r = 0; r < nr; ++r) ibar_d[r] = ibar_in[r] * sc;
  out_mul[0] = 1.0 / (scale_g * sc);
}

// true when every value is finite (flag stays 1)
static __global__ void finite_kernel(const double* __restrict__ x, long long n, int* __restrict__ flag) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    if (!isfinite(x[q])) *flag = 0;
}

}  // namespace pn
