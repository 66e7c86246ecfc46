// Preprocessing on the GPU: template/mask generation from atoms (Gaussian
// splat, ball dilation), the periodic Laplace filter and core-weight erosion.
// These run once per search; they mirror the reference's host helpers:
//   _powerfit.pyx:75-140   blur_points       (Gaussian splat, 4 sigma cut-off)
//   _powerfit.pyx:143-206  dilate_points     (balls of given radii)
//   powerfitter.py:212-215 scipy.ndimage.laplace(mode='wrap')
//   helpers.py:26-34       determine_core_indices (repeated binary erosion)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "../../include/powerfit_gb300.h"

namespace {

thread_local char g_prep_err[256] = "";

int prep_fail(int code, const char* what, cudaError_t e) {
  snprintf(g_prep_err, sizeof(g_prep_err), "%s: %s", what, cudaGetErrorString(e));
  return code;
}

struct Grid3 {
  int nz, ny, nx;
};

// Box bounds of one point (reference _powerfit.pyx:117-131 / :185-197): the box
// [ceil(p - e), floor(p + e)] clipped below at -(n-1) with wraparound (0
// without) and above at n-1; negative indices wrap once.
__device__ __forceinline__ void box(double p, double e, int n, bool wrap, int& lo, int& hi) {
  lo = (int)ceil(p - e);
  hi = (int)floor(p + e);
  lo = max(lo, wrap ? -(n - 1) : 0);
  hi = min(hi, n - 1);
}

// one block per point; threads stride over the point's box
__global__ void k_blur_points(const double* __restrict__ pts, const double* __restrict__ w, long long n,
                              double sigma, double* __restrict__ out, Grid3 g, int wrap) {
  const long long i = blockIdx.x;
  if (i >= n) return;
  const double px = pts[i], py = pts[n + i], pz = pts[2 * n + i];
  const double e = 4.0 * sigma, e2 = e * e, ds2 = 2.0 * sigma * sigma;
  int x0, x1, y0, y1, z0, z1;
  box(px, e, g.nx, wrap, x0, x1);
  box(py, e, g.ny, wrap, y0, y1);
  box(pz, e, g.nz, wrap, z0, z1);
  const int wx = x1 - x0 + 1, wy = y1 - y0 + 1, wz = z1 - z0 + 1;
  if (wx <= 0 || wy <= 0 || wz <= 0) return;
  const long long cnt = (long long)wx * wy * wz;
  for (long long k = threadIdx.x; k < cnt; k += blockDim.x) {
    const int x = x0 + (int)(k % wx);
    const int y = y0 + (int)((k / wx) % wy);
    const int z = z0 + (int)(k / ((long long)wx * wy));
    const double dz = z - pz, dy = y - py, dx = x - px;
    const double d2 = (dx * dx + dy * dy) + dz * dz;
    if (d2 <= e2) {
      const int ix = x < 0 ? x + g.nx : x, iy = y < 0 ? y + g.ny : y, iz = z < 0 ? z + g.nz : z;
      atomicAdd(out + ((long long)iz * g.ny + iy) * g.nx + ix, w[i] * exp(-d2 / ds2));
    }
  }
}

__global__ void k_dilate_points(const double* __restrict__ pts, const double* __restrict__ radii, long long n,
                                double* __restrict__ out, Grid3 g, int wrap) {
  const long long i = blockIdx.x;
  if (i >= n) return;
  const double px = pts[i], py = pts[n + i], pz = pts[2 * n + i];
  const double r = radii[i], r2 = r * r;
  int x0, x1, y0, y1, z0, z1;
  box(px, r, g.nx, wrap, x0, x1);
  box(py, r, g.ny, wrap, y0, y1);
  box(pz, r, g.nz, wrap, z0, z1);
  const int wx = x1 - x0 + 1, wy = y1 - y0 + 1, wz = z1 - z0 + 1;
  if (wx <= 0 || wy <= 0 || wz <= 0) return;
  const long long cnt = (long long)wx * wy * wz;
  for (long long k = threadIdx.x; k < cnt; k += blockDim.x) {
    const int x = x0 + (int)(k % wx);
    const int y = y0 + (int)((k / wx) % wy);
    const int z = z0 + (int)(k / ((long long)wx * wy));
    const double dz = z - pz, dy = y - py, dx = x - px;
    if ((dx * dx + dy * dy) + dz * dz <= r2) {
      const int ix = x < 0 ? x + g.nx : x, iy = y < 0 ? y + g.ny : y, iz = z < 0 ? z + g.nz : z;
      out[((long long)iz * g.ny + iy) * g.nx + ix] = 1.0;
    }
  }
}

// scipy.ndimage.laplace(mode='wrap'): sum over axes of x[i-1] - 2 x[i] + x[i+1]
// (axis 0 first, as the filter accumulates axis by axis)
__global__ void k_laplace_wrap(const double* __restrict__ a, double* __restrict__ o, Grid3 g) {
  const long long n = (long long)g.nz * g.ny * g.nx;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % g.nx), y = (int)((i / g.nx) % g.ny), z = (int)(i / ((long long)g.nx * g.ny));
    const long long sz = (long long)g.ny * g.nx;
    const double c = a[i];
    const double zm = a[i + ((z == 0) ? (g.nz - 1) * sz : -sz)], zp = a[i + ((z == g.nz - 1) ? -(g.nz - 1) * sz : sz)];
    const double ym = a[i + ((y == 0) ? (long long)(g.ny - 1) * g.nx : -g.nx)];
    const double yp = a[i + ((y == g.ny - 1) ? -(long long)(g.ny - 1) * g.nx : g.nx)];
    const double xm = a[i + ((x == 0) ? g.nx - 1 : -1)], xp = a[i + ((x == g.nx - 1) ? -(g.nx - 1) : 1)];
    const double lz = zm - 2.0 * c + zp;
    const double ly = ym - 2.0 * c + yp;
    const double lx = xm - 2.0 * c + xp;
    o[i] = (lz + ly) + lx;
  }
}

// one binary erosion with the 6-connected cross, border value 0 (scipy
// binary_erosion defaults); counts surviving voxels and adds them to core
__global__ void k_erode(const unsigned char* __restrict__ in, unsigned char* __restrict__ out,
                        double* __restrict__ core, Grid3 g, unsigned long long* __restrict__ alive) {
  const long long n = (long long)g.nz * g.ny * g.nx;
  unsigned long long local = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % g.nx), y = (int)((i / g.nx) % g.ny), z = (int)(i / ((long long)g.nx * g.ny));
    const long long sz = (long long)g.ny * g.nx;
    unsigned char v = in[i];
    if (v) {
      v = (x > 0 && in[i - 1]) && (x < g.nx - 1 && in[i + 1]) && (y > 0 && in[i - g.nx]) &&
          (y < g.ny - 1 && in[i + g.nx]) && (z > 0 && in[i - sz]) && (z < g.nz - 1 && in[i + sz]);
    }
    out[i] = v;
    if (v) {
      core[i] += 1.0;
      ++local;
    }
  }
  if (local) atomicAdd(alive, local);
}

__global__ void k_seed_core(const double* __restrict__ mask, unsigned char* __restrict__ er, double* __restrict__ core,
                            long long n, unsigned long long* __restrict__ alive) {
  unsigned long long local = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const bool v = mask[i] > 0;
    er[i] = v;
    core[i] = v ? 1.0 : 0.0;
    local += v;
  }
  if (local) atomicAdd(alive, local);
}

template <class T>
struct DevBuf {
  T* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) { return cudaMalloc((void**)&p, n * sizeof(T)); }
};

bool bad_grid(int nz, int ny, int nx) { return nz < 1 || ny < 1 || nx < 1; }

}  // namespace

extern "C" {

int pf_prep_error(char* buf, size_t len) {
  if (!buf || !len) return PF_E_ARG;
  snprintf(buf, len, "%s", g_prep_err);
  return PF_OK;
}

int pf_blur_points(const double* points, const double* weights, int64_t n, double sigma, double* out, int nz,
                   int ny, int nx, int wraparound) {
  if (!points || !weights || !out || n < 0 || bad_grid(nz, ny, nx) || !(sigma > 0)) {
    snprintf(g_prep_err, sizeof(g_prep_err), "pf_blur_points: bad arguments");
    return PF_E_ARG;
  }
  const size_t N = (size_t)nz * ny * nx;
  DevBuf<double> dp, dw, dout;
  cudaError_t e = dp.alloc(3 * (size_t)std::max<int64_t>(n, 1));
  if (e == cudaSuccess) e = dw.alloc((size_t)std::max<int64_t>(n, 1));
  if (e == cudaSuccess) e = dout.alloc(N);
  if (e != cudaSuccess) return prep_fail(PF_E_NOMEM, "blur_points allocation", e);
  if (n > 0) {
    e = cudaMemcpy(dp.p, points, 3 * n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dw.p, weights, n * sizeof(double), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemcpy(dout.p, out, N * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n > 0) {
    k_blur_points<<<(unsigned)n, 256>>>(dp.p, dw.p, n, sigma, dout.p, Grid3{nz, ny, nx}, wraparound ? 1 : 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, dout.p, N * sizeof(double), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? PF_OK : prep_fail(PF_E_CUDA, "blur_points", e);
}

int pf_dilate_points(const double* points, const double* radii, int64_t n, double* out, int nz, int ny, int nx,
                     int wraparound) {
  if (!points || !radii || !out || n < 0 || bad_grid(nz, ny, nx)) {
    snprintf(g_prep_err, sizeof(g_prep_err), "pf_dilate_points: bad arguments");
    return PF_E_ARG;
  }
  const size_t N = (size_t)nz * ny * nx;
  DevBuf<double> dp, dr, dout;
  cudaError_t e = dp.alloc(3 * (size_t)std::max<int64_t>(n, 1));
  if (e == cudaSuccess) e = dr.alloc((size_t)std::max<int64_t>(n, 1));
  if (e == cudaSuccess) e = dout.alloc(N);
  if (e != cudaSuccess) return prep_fail(PF_E_NOMEM, "dilate_points allocation", e);
  if (n > 0) {
    e = cudaMemcpy(dp.p, points, 3 * n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dr.p, radii, n * sizeof(double), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemcpy(dout.p, out, N * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n > 0) {
    k_dilate_points<<<(unsigned)n, 256>>>(dp.p, dr.p, n, dout.p, Grid3{nz, ny, nx}, wraparound ? 1 : 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, dout.p, N * sizeof(double), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? PF_OK : prep_fail(PF_E_CUDA, "dilate_points", e);
}

int pf_laplace_wrap(const double* in, double* out, int nz, int ny, int nx) {
  if (!in || !out || bad_grid(nz, ny, nx)) {
    snprintf(g_prep_err, sizeof(g_prep_err), "pf_laplace_wrap: bad arguments");
    return PF_E_ARG;
  }
  const size_t N = (size_t)nz * ny * nx;
  DevBuf<double> a, o;
  cudaError_t e = a.alloc(N);
  if (e == cudaSuccess) e = o.alloc(N);
  if (e != cudaSuccess) return prep_fail(PF_E_NOMEM, "laplace allocation", e);
  e = cudaMemcpy(a.p, in, N * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_laplace_wrap<<<(unsigned)std::min<size_t>((N + 255) / 256, 8192), 256>>>(a.p, o.p, Grid3{nz, ny, nx});
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, o.p, N * sizeof(double), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? PF_OK : prep_fail(PF_E_CUDA, "laplace", e);
}

int pf_core_indices(const double* mask, double* out, int nz, int ny, int nx) {
  if (!mask || !out || bad_grid(nz, ny, nx)) {
    snprintf(g_prep_err, sizeof(g_prep_err), "pf_core_indices: bad arguments");
    return PF_E_ARG;
  }
  const size_t N = (size_t)nz * ny * nx;
  DevBuf<double> m, core;
  DevBuf<unsigned char> e0, e1;
  DevBuf<unsigned long long> alive;
  cudaError_t e = m.alloc(N);
  if (e == cudaSuccess) e = core.alloc(N);
  if (e == cudaSuccess) e = e0.alloc(N);
  if (e == cudaSuccess) e = e1.alloc(N);
  if (e == cudaSuccess) e = alive.alloc(1);
  if (e != cudaSuccess) return prep_fail(PF_E_NOMEM, "core_indices allocation", e);
  e = cudaMemcpy(m.p, mask, N * sizeof(double), cudaMemcpyHostToDevice);
  const unsigned blocks = (unsigned)std::min<size_t>((N + 255) / 256, 8192);
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemset(alive.p, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) {
    k_seed_core<<<blocks, 256>>>(m.p, e0.p, core.p, (long long)N, alive.p);
    e = cudaMemcpy(&h, alive.p, sizeof(h), cudaMemcpyDeviceToHost);
  }
  // erode until nothing survives (at most min(shape)/2 + 1 rounds)
  const int max_rounds = std::min(nz, std::min(ny, nx)) / 2 + 2;
  for (int round = 0; e == cudaSuccess && h > 0 && round < max_rounds; ++round) {
    e = cudaMemset(alive.p, 0, sizeof(unsigned long long));
    if (e != cudaSuccess) break;
    k_erode<<<blocks, 256>>>(e0.p, e1.p, core.p, Grid3{nz, ny, nx}, alive.p);
    e = cudaMemcpy(&h, alive.p, sizeof(h), cudaMemcpyDeviceToHost);
    std::swap(e0.p, e1.p);
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, core.p, N * sizeof(double), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? PF_OK : prep_fail(PF_E_CUDA, "core_indices", e);
}

}  // extern "C"
