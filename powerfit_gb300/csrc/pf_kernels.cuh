// Kernels of the exhaustive 6D LCC search (sm_103a).
//
// Rotations are processed in pairs.  For a pair (a, b) three complex fields
// are formed from the rotated template t and mask m (the rotation follows the
// reference rotate_grid3d, _extensions.c:7-196):
//     f0 = t_a - i m_a,   f1 = t_b - i m_b,   f2 = m_a^2 - i m_b^2
// Their spectra F give, after conj(F) * FT(target) or FT(target^2) and an
// inverse transform (powerfitter.py:349-373 computes the same correlations
// with six real transforms per rotation):
//     IFFT(conj(F0) S1) = gcc_a + i ave_a,  IFFT(conj(F1) S1) = gcc_b + i ave_b,
//     IFFT(conj(F2) S2) = ave2_a + i ave2_b
// with S1 = FT(target')/N and S2 = FT(target'^2)/N.
//
// Three passes per batch of pairs, intermediate spectra laid out
// buf[pair][field][kx][z][y] (complex float32):
//   pass 1  per (pair, z, y-tile): rotate/gather, forward x transform, store
//           transposed so that pass 2 reads contiguous (z, y) planes;
//   pass 2  per (pair, field, kx): forward y and z transforms of the (z, y)
//           plane in shared memory, conj product with the target spectrum,
//           inverse z and y transforms, store in place;
//   pass 3  per (z, y-tile), looping over the batch's pairs: inverse x
//           transform, LCC normalisation, running max / argmax kept in
//           registers for the whole batch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pf_fft.cuh"
#include "pf_fft_mma.cuh"
#include "pf_fft_tc05.cuh"

namespace pf {

constexpr int kEmax = 16;          // complex values a thread holds per stage chunk
constexpr int kThreadsLine = 256;  // pass 1 / pass 3 / target x transform
constexpr int kThreadsPlane = 512; // pass 2 / target (y, z) transform
// resident pass-1 blocks per SM that the register allocation must allow (0: compiler's choice)
#ifndef PF_PASS1_MIN_BLOCKS
#define PF_PASS1_MIN_BLOCKS 4
#endif
#if PF_PASS1_MIN_BLOCKS > 0
#define PF_PASS1_BOUNDS __launch_bounds__(kThreadsLine, PF_PASS1_MIN_BLOCKS)
#else
#define PF_PASS1_BOUNDS __launch_bounds__(kThreadsLine)
#endif
constexpr int kPad = 1;            // shared-memory row padding (complex) for conflict-free access

// 32.32 fixed-point rotation matrix (row-major R, element r_i = round(R_i * 2^32))
struct RotFixed {
  long long r[9];
};

struct Geometry {
  int nz, ny, nx;
  int rmax;     // sphere radius of the rotation (min(shape)//2)
  int reff;     // radius outside which rotated template and mask are known to be zero
  int nvz;      // number of z planes holding data after rotation (|cz| <= min(rmax, reff))
  int zlo;      // planes 0..zlo and nz-(nvz-zlo-1)..nz-1 hold data
};

__device__ __forceinline__ int signed_coord(int i, int n) {
  // output voxel i of an axis of size n corresponds to offset i (i <= n/2) or i - n;
  // for even n the voxel n/2 takes the +n/2 offset (written last by the reference loops)
  return (2 * i <= n) ? i : i - n;
}

__device__ __forceinline__ int valid_plane(const Geometry& g, int zi) {
  return (zi <= g.zlo) ? zi : g.nz - g.nvz + zi;
}

__device__ __forceinline__ int wrap1(int i, int n) {
  // periodic index; rotation matrices keep i within [-n, 2n), any other
  // matrix still lands inside the grid
  if (i >= 0 && i < n) return i;
  if (i < 0 && i >= -n) return i + n;
  if (i >= n && i < 2 * n) return i - n;
  const int r = i % n;
  return r < 0 ? r + n : r;
}

// ---------------------------------------------------------------------------
// Rotation gather (reference rotate_grid3d, _extensions.c:55-180)
// ---------------------------------------------------------------------------
// source point q = R^T p in 32.32 fixed point: q_x = r0 x + r3 y + r6 z, etc.
struct SourcePoint {
  long long qx, qy, qz;
};

__device__ __forceinline__ SourcePoint source_point(const RotFixed& R, int cz, int cy, int cx) {
  SourcePoint s;
  s.qx = R.r[6] * cz + R.r[3] * cy + R.r[0] * cx;
  s.qy = R.r[7] * cz + R.r[4] * cy + R.r[1] * cx;
  s.qz = R.r[8] * cz + R.r[5] * cy + R.r[2] * cx;
  return s;
}

// C round() (halves away from zero) of a 32.32 fixed-point value.  Values
// within 2^-23 of a half are decided in float64 with the reference's operation
// order (((r6 z) + (r3 y)) + (r0 x), no fused multiply-add), so that the nearest
// voxel agrees with the float64 reference even when the fixed-point
// representation of the matrix is 2^-33 away from its float64 value.
// The float64 decision is a separate, never-inlined function: inlined, the
// compiler evaluates it under a predicate for every point, and GB300 issues
// float64 at 1/64 of the float32 rate.
static __device__ __noinline__ int round_f64(const double* __restrict__ rd, int c0, int c1, int c2, int cz, int cy, int cx) {
  const double v = __dadd_rn(__dadd_rn(__dmul_rn(rd[c2], (double)cz), __dmul_rn(rd[c1], (double)cy)),
                             __dmul_rn(rd[c0], (double)cx));
  return (int)round(v);
}

__device__ __forceinline__ int round_fixed(long long q, const double* __restrict__ rd, int c0, int c1, int c2,
                                           int cz, int cy, int cx) {
  const long long fl = q >> 32;
  const unsigned int frac = (unsigned int)(q & 0xffffffffLL);
  const int dist = (int)(frac - 0x80000000u);
  if (dist > 512 || dist < -512) return (int)fl + (frac > 0x80000000u ? 1 : 0);
  return round_f64(rd, c0, c1, c2, cz, cy, cx);
}

// 0.32 fixed-point fraction -> float in [0, 1): the top 23 bits become the
// mantissa of a float in [1, 2), minus 1 (exact; integer ops instead of a
// conversion instruction)
__device__ __forceinline__ float frac_to_float(unsigned int f) {
  return __int_as_float(0x3f800000u | (f >> 9)) - 1.0f;
}

struct GatherSrc {
  const float* __restrict__ tmpl;   // template, float32, C order (z, y, x)
  const float* __restrict__ mask;   // mask, float32
  const float2* __restrict__ tmpl_pairs = nullptr;  // (t[z][y][x], t[z][y][x+1 wrapped]) per voxel
};

// trilinear template value and nearest mask value at rotated offset p
__device__ __forceinline__ void gather_point(const Geometry& g, const GatherSrc& src, const RotFixed& R,
                                             const double* __restrict__ rd, int cz, int cy, int cx,
                                             float& t, float& m) {
  const SourcePoint s = source_point(R, cz, cy, cx);
  const long long sxy = (long long)g.nx * g.ny;
  // trilinear (x, then y, then z, as the reference)
  {
    const int x0 = (int)(s.qx >> 32), y0 = (int)(s.qy >> 32), z0 = (int)(s.qz >> 32);
    const float fx = frac_to_float((unsigned int)s.qx);
    const float fy = frac_to_float((unsigned int)s.qy);
    const float fz = frac_to_float((unsigned int)s.qz);
    const int ix0 = wrap1(x0, g.nx), ix1 = wrap1(x0 + 1, g.nx);
    const long long iy0 = (long long)wrap1(y0, g.ny) * g.nx, iy1 = (long long)wrap1(y0 + 1, g.ny) * g.nx;
    const long long iz0 = (long long)wrap1(z0, g.nz) * sxy, iz1 = (long long)wrap1(z0 + 1, g.nz) * sxy;
    if (!(PF_CHECK(kChkGather, ix0, g.nx) & PF_CHECK(kChkGather, ix1, g.nx) & PF_CHECK(kChkGather, iy0, sxy) &
          PF_CHECK(kChkGather, iy1, sxy) & PF_CHECK(kChkGather, iz0, sxy * g.nz) & PF_CHECK(kChkGather, iz1, sxy * g.nz))) {
      t = m = 0.f;
      return;
    }
    const float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
    const float* T = src.tmpl;
    const float c00 = __ldg(T + iz0 + iy0 + ix0) * gx + __ldg(T + iz0 + iy0 + ix1) * fx;
    const float c10 = __ldg(T + iz0 + iy1 + ix0) * gx + __ldg(T + iz0 + iy1 + ix1) * fx;
    const float c01 = __ldg(T + iz1 + iy0 + ix0) * gx + __ldg(T + iz1 + iy0 + ix1) * fx;
    const float c11 = __ldg(T + iz1 + iy1 + ix0) * gx + __ldg(T + iz1 + iy1 + ix1) * fx;
    const float c0 = c00 * gy + c10 * fy;
    const float c1 = c01 * gy + c11 * fy;
    t = c0 * gz + c1 * fz;
  }
  // nearest
  {
    const int x0 = round_fixed(s.qx, rd, 0, 3, 6, cz, cy, cx);
    const int y0 = round_fixed(s.qy, rd, 1, 4, 7, cz, cy, cx);
    const int z0 = round_fixed(s.qz, rd, 2, 5, 8, cz, cy, cx);
    const long long i = (long long)wrap1(z0, g.nz) * sxy + (long long)wrap1(y0, g.ny) * g.nx + wrap1(x0, g.nx);
    m = PF_CHECK(kChkGather, i, sxy * g.nz) ? __ldg(src.mask + i) : 0.f;
  }
}

#ifdef PF_GENERIC_KERNELS
// tmpl_pairs[i] = (t[i], t[i with x + 1 wrapped])
__global__ void k_make_pairs(const float* __restrict__ t, float2* __restrict__ out, int nx, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx);
    out[i] = make_float2(t[i], t[x + 1 < nx ? i + 1 : i + 1 - nx]);
  }
}
#endif  // PF_GENERIC_KERNELS

// ---------------------------------------------------------------------------
// Pass 1: gather + forward x transform, store buf[pair][f][kx][z][y]
// ---------------------------------------------------------------------------
struct Pass1Params {
  Geometry g;
  AxisPlan px;
  GatherSrc src;
  const float2* __restrict__ twx;       // x twiddles (nx entries)
  const RotFixed* __restrict__ rots;    // fixed-point matrices of this scan
  const double* __restrict__ rotd;      // float64 matrices (9 per rotation)
  long long first_rot;                  // rotation index of pair 0, rotation a
  long long nrot;                       // total rotations of this scan
  float2* __restrict__ buf;             // intermediate spectra
  int ty;                               // rows per tile
  const int4* __restrict__ rows;        // fast path: (z, y, points in the sphere, 0) of every reachable row
  int nrows;
  long long buf_len = 0;                // elements of buf (bounds checks)
};

struct TransposedStore {  // line = f*ty + r  (row y0 + r of field f); idx = kx
  float2* base;           // buf + pair offset
  int ty, y0, ny, nz, nx, z;
  long long lim;          // elements from base on (bounds checks)
  __device__ __forceinline__ void store(int line, int idx, float2 v) const {
    const int f = line / ty, r = line - f * ty;
    const int y = y0 + r;
    const long long i = (((long long)f * nx + idx) * nz + z) * ny + y;
    if (y < ny && PF_CHECK(kChkBufStore, i, lim)) base[i] = v;
  }
};

#ifdef PF_GENERIC_KERNELS
// TC (here and below): DFT stages in split-bf16x3 on the tensor cores (pf_fft_mma.cuh)
template <bool TC>
__global__ void __launch_bounds__(kThreadsLine) k_pass1(const Pass1Params p) {
  extern __shared__ float2 sm[];
  const Geometry& g = p.g;
  const int X = g.nx;
  float2* tw = sm;
  float2* fld = sm + X;                      // [3][ty][X + kPad]
  const int rs = X + kPad;
  for (int i = threadIdx.x; i < X; i += blockDim.x) tw[i] = p.twx[i];

  const int z = valid_plane(g, blockIdx.x);
  const int cz = signed_coord(z, g.nz);
  const int y0 = blockIdx.y * p.ty;
  const int pair = blockIdx.z;
  const long long ra = p.first_rot + 2LL * pair, rb = ra + 1;
  const bool has_a = ra < p.nrot, has_b = rb < p.nrot;
  const RotFixed Ra = p.rots[has_a ? ra : 0];
  const RotFixed Rb = p.rots[has_b ? rb : 0];
  const double* rda = p.rotd + 9 * (has_a ? ra : 0);
  const double* rdb = p.rotd + 9 * (has_b ? rb : 0);
  const int r2 = min(g.rmax, g.reff) * min(g.rmax, g.reff);

  for (int v = threadIdx.x; v < p.ty * X; v += blockDim.x) {
    const int r = v / X, x = v - r * X;
    const int y = y0 + r;
    float ta = 0.f, ma = 0.f, tb = 0.f, mb = 0.f;
    if (y < g.ny) {
      const int cy = signed_coord(y, g.ny), cx = signed_coord(x, X);
      if (cz * cz + cy * cy + cx * cx <= r2) {
        if (has_a) gather_point(g, p.src, Ra, rda, cz, cy, cx, ta, ma);
        if (has_b) gather_point(g, p.src, Rb, rdb, cz, cy, cx, tb, mb);
      }
    }
    if (PF_CHECK_SMEM(kChkSmem, fld + (2 * p.ty + r) * rs + x, 8)) {
      fld[(0 * p.ty + r) * rs + x] = make_float2(ta, -ma);
      fld[(1 * p.ty + r) * rs + x] = make_float2(tb, -mb);
      fld[(2 * p.ty + r) * rs + x] = make_float2(ma * ma, -(mb * mb));
    }
  }
  __syncthreads();

  SmemLines lines{fld, rs, 1};
  const long long pair_off = (long long)pair * 3 * g.nx * g.nz * g.ny;
  TransposedStore out{p.buf + pair_off, p.ty, y0, g.ny, g.nz, g.nx, z, p.buf_len - pair_off};
  fft_lines<false, kEmax, TC>(p.px, 3 * p.ty, tw, lines, lines, out, true, false);
}

#endif  // PF_GENERIC_KERNELS

// ---------------------------------------------------------------------------
// Pass 2: per (pair, field, kx) plane: y, z forward, product, z, y inverse
// ---------------------------------------------------------------------------
struct Pass2Params {
  Geometry g;
  AxisPlan py, pz;
  const float2* __restrict__ twy;
  const float2* __restrict__ twz;
  float2* __restrict__ buf;
  const float2* __restrict__ s1;  // FT(target')/N   layout [kx][kz][ky]
  const float2* __restrict__ s2;  // FT(target'^2)/N layout [kx][kz][ky]
  int nfield;                     // fields per pair in buf (3)
  int mode;                       // 0: correlate (full), 1: forward only -> out
  float2* __restrict__ out;       // mode 1: spectra, layout [f][kx][kz][ky]
  float scale;                    // mode 1: multiply spectra by this
  long long buf_len = 0;          // elements of buf, of s1 and of s2, of out (bounds checks)
  long long spec_len = 0;
  long long out_len = 0;
};

struct RowMapLines {  // line l -> data row (valid planes only), element idx along y
  float2* base;
  int rs, zlo, shift;
  __device__ __forceinline__ int row(int l) const { return l <= zlo ? l : l + shift; }
  __device__ __forceinline__ float2 load(int line, int idx) const {
    const float2* q = base + row(line) * rs + idx;
    return PF_CHECK_SMEM(kChkSmem, q, 8) ? *q : make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ void store(int line, int idx, float2 v) const {
    float2* q = base + row(line) * rs + idx;
    if (PF_CHECK_SMEM(kChkSmem, q, 8)) *q = v;
  }
};

struct ProductStore {  // column transforms: line = ky, idx = kz
  float2* base;
  int rs;
  const float2* __restrict__ spec;  // [kz][ky] plane of the target spectrum for this kx
  int ny;
  long long lim;                    // elements from spec on (bounds checks)
  __device__ __forceinline__ void store(int line, int idx, float2 v) const {
    const long long i = (long long)idx * ny + line;
    float2* q = base + idx * rs + line;
    if (PF_CHECK(kChkSpectrum, i, lim) && PF_CHECK_SMEM(kChkSmem, q, 8)) *q = cmulc(v, __ldg(spec + i));
  }
};

// Shared memory of the tcgen05 plane pass: the plane (plane_smem), then the
// operand area of the tensor-core stages on a 1024-byte boundary.
__host__ __device__ inline size_t pass2_tc05_smem(size_t plane_bytes) {
  return plane_bytes + 1024 + kTc05SmemBytes;
}

#ifdef PF_GENERIC_KERNELS
// TC: 0 float32 stages; 1 split-bf16x3 mma.sync stages; 2 split-bf16x3
// tcgen05 stages (operands in shared memory after the plane)
template <int TC>
__global__ void __launch_bounds__(kThreadsPlane) k_pass2(const Pass2Params p) {
  extern __shared__ float2 sm[];
  const Geometry& g = p.g;
  const int Y = g.ny, Z = g.nz;
  float2* twy = sm;
  float2* twz = sm + Y;
  float2* pl = sm + Y + Z;                      // [Z][Y + kPad]
  const int rs = Y + kPad;
  for (int i = threadIdx.x; i < Y; i += blockDim.x) twy[i] = p.twy[i];
  for (int i = threadIdx.x; i < Z; i += blockDim.x) twz[i] = p.twz[i];
  if constexpr (TC == 2) {
    static_assert(kThreadsPlane == kTc05Threads, "the tcgen05 stages map one item per thread of the plane pass");
    const size_t plane_end = (size_t)(Y + Z + (size_t)Z * rs) * sizeof(float2);
    const unsigned int base = smem_u32(sm);
    const unsigned int ops = (base + (unsigned int)plane_end + 1023u) & ~1023u;
    tc05_begin(reinterpret_cast<char*>(sm) + (ops - base));
  }

  const int kx = blockIdx.x, f = blockIdx.y, pair = blockIdx.z;
  const long long plane = (long long)Z * Y;
  const long long plane_off = (((long long)pair * p.nfield + f) * g.nx + kx) * plane;
  float2* gplane = p.buf + plane_off;
  const long long glim = p.buf_len - plane_off;

  // load valid rows, zero the rest
  const int nvz = g.nvz;
  for (int v = threadIdx.x; v < Z * Y; v += blockDim.x) {
    const int z = v / Y, y = v - z * Y;
    const long long i = (long long)z * Y + y;
    const bool valid = (z <= g.zlo) || (z >= Z - (nvz - g.zlo - 1));
    if (PF_CHECK_SMEM(kChkSmem, pl + z * rs + y, 8))
      pl[z * rs + y] = valid && PF_CHECK(kChkBufLoad, i, glim) ? gplane[i] : make_float2(0.f, 0.f);
  }
  __syncthreads();

  RowMapLines rows{pl, rs, g.zlo, Z - nvz};
  fft_lines<false, kEmax, TC>(p.py, nvz, twy, rows, rows, rows, true, true);
  SmemLines cols{pl, 1, rs};
  if (p.mode == 0) {
    const float2* spec = (f == p.nfield - 1 ? p.s2 : p.s1) + (long long)kx * plane;
    ProductStore prod{pl, rs, spec, Y, p.spec_len - (long long)kx * plane};
    fft_lines<false, kEmax, TC>(p.pz, Y, twz, cols, cols, prod, true, true);
    fft_lines<true, kEmax, TC>(p.pz, Y, twz, cols, cols, cols, true, true);
    SmemLines allrows{pl, rs, 1};
    fft_lines<true, kEmax, TC>(p.py, Z, twy, allrows, allrows, allrows, true, true);
    for (int v = threadIdx.x; v < Z * Y; v += blockDim.x) {
      const int z = v / Y, y = v - z * Y;
      const long long i = (long long)z * Y + y;
      if (PF_CHECK(kChkBufStore, i, glim) && PF_CHECK_SMEM(kChkSmem, pl + z * rs + y, 8)) gplane[i] = pl[z * rs + y];
    }
    if constexpr (TC == 2) tc05_end();
  } else {
    fft_lines<false, kEmax, TC>(p.pz, Y, twz, cols, cols, cols, true, true);
    const long long out_off = ((long long)f * g.nx + kx) * plane;
    float2* o = p.out + out_off;
    for (int v = threadIdx.x; v < Z * Y; v += blockDim.x) {
      const int z = v / Y, y = v - z * Y;
      const long long i = (long long)z * Y + y;
      if (PF_CHECK(kChkOut, i, p.out_len - out_off) && PF_CHECK_SMEM(kChkSmem, pl + z * rs + y, 8))
        o[i] = cscale(pl[z * rs + y], p.scale);
    }
    if constexpr (TC == 2) tc05_end();
  }
}

#endif  // PF_GENERIC_KERNELS

// ---------------------------------------------------------------------------
// Pass 2, split form for (z, y) planes larger than shared memory (e.g. 192^3):
//   2a  y transforms of tiles of rows (forward: valid planes only),
//   2b  per tile of y columns: z forward, conj product (or forward only),
//       z inverse,
//   2c  inverse y transforms of tiles of rows.
// The planes go through global memory between the steps.
// ---------------------------------------------------------------------------
struct SplitRowsParams {
  Geometry g;
  AxisPlan py;
  const float2* __restrict__ twy;
  float2* __restrict__ buf;
  int nfield;
  int rows_per_tile;
  int inverse;     // 0: forward, valid z rows only; 1: inverse, all rows
  long long buf_len = 0;          // elements of buf (bounds checks)
};

struct SplitColsParams {
  Geometry g;
  AxisPlan pz;
  const float2* __restrict__ twz;
  float2* __restrict__ buf;
  const float2* __restrict__ s1;
  const float2* __restrict__ s2;
  int nfield;
  int cols_per_tile;
  int mode;                       // 0: z forward, product, z inverse; 1: z forward only -> out
  float2* __restrict__ out;
  float scale;
  long long buf_len = 0;          // elements of buf, of s1 and of s2, of out (bounds checks)
  long long spec_len = 0;
  long long out_len = 0;
};

#ifdef PF_GENERIC_KERNELS
// grid: (row tiles of one (field, kx) plane, kx, pair * nfield + field)
template <bool TC>
__global__ void __launch_bounds__(kThreadsLine) k_split_rows(const SplitRowsParams p) {
  extern __shared__ float2 sm[];
  const Geometry& g = p.g;
  const int Y = g.ny, Z = g.nz;
  float2* tw = sm;
  float2* t = sm + Y;                           // [rows][Y + kPad]
  const int rs = Y + kPad;
  for (int i = threadIdx.x; i < Y; i += blockDim.x) tw[i] = p.twy[i];
  const int nrow_all = p.inverse ? Z : g.nvz;
  const int r0 = blockIdx.x * p.rows_per_tile;
  const int nr = min(p.rows_per_tile, nrow_all - r0);
  if (nr <= 0) return;
  const int kx = blockIdx.y;
  const long long plane_off = ((long long)blockIdx.z * g.nx + kx) * ((long long)Z * Y);
  float2* gplane = p.buf + plane_off;
  const long long glim = p.buf_len - plane_off;
  auto row_of = [&](int l) { const int i = r0 + l; return (p.inverse || i <= g.zlo) ? i : i + Z - g.nvz; };
  for (int v = threadIdx.x; v < nr * Y; v += blockDim.x) {
    const int l = v / Y, y = v - l * Y;
    const long long i = (long long)row_of(l) * Y + y;
    if (PF_CHECK_SMEM(kChkSmem, t + l * rs + y, 8))
      t[l * rs + y] = PF_CHECK(kChkBufLoad, i, glim) ? gplane[i] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  SmemLines lines{t, rs, 1};
  if (p.inverse) fft_lines<true, kEmax, TC>(p.py, nr, tw, lines, lines, lines, true, true);
  else fft_lines<false, kEmax, TC>(p.py, nr, tw, lines, lines, lines, true, true);
  for (int v = threadIdx.x; v < nr * Y; v += blockDim.x) {
    const int l = v / Y, y = v - l * Y;
    const long long i = (long long)row_of(l) * Y + y;
    if (PF_CHECK(kChkBufStore, i, glim) && PF_CHECK_SMEM(kChkSmem, t + l * rs + y, 8)) gplane[i] = t[l * rs + y];
  }
}

// grid: (column tiles, kx, pair * nfield + field)
template <bool TENSOR>
__global__ void __launch_bounds__(kThreadsLine) k_split_cols(const SplitColsParams p) {
  extern __shared__ float2 sm[];
  const Geometry& g = p.g;
  const int Y = g.ny, Z = g.nz;
  const int TC = p.cols_per_tile;
  float2* tw = sm;
  float2* t = sm + Z;                           // [Z][TC + kPad]
  const int rs = TC + kPad;
  for (int i = threadIdx.x; i < Z; i += blockDim.x) tw[i] = p.twz[i];
  const int y0 = blockIdx.x * TC;
  const int nc = min(TC, Y - y0);
  const int kx = blockIdx.y;
  const int pf = blockIdx.z;
  const int f = pf % p.nfield;
  const long long plane = (long long)Z * Y;
  const long long plane_off = ((long long)pf * g.nx + kx) * plane;
  float2* gplane = p.buf + plane_off;
  const long long glim = p.buf_len - plane_off;
  const int nvz = g.nvz;
  for (int v = threadIdx.x; v < Z * TC; v += blockDim.x) {
    const int z = v / TC, c = v - z * TC;
    const long long i = (long long)z * Y + y0 + c;
    const bool valid = c < nc && (p.mode == 1 || z <= g.zlo || z >= Z - (nvz - g.zlo - 1));
    if (PF_CHECK_SMEM(kChkSmem, t + z * rs + c, 8))
      t[z * rs + c] = valid && PF_CHECK(kChkBufLoad, i, glim) ? gplane[i] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  SmemLines cols{t, 1, rs};
  if (p.mode == 0) {
    const long long spec_off = (long long)kx * plane + y0;
    const float2* spec = (f == p.nfield - 1 ? p.s2 : p.s1) + spec_off;
    ProductStore prod{t, rs, spec, Y, p.spec_len - spec_off};
    fft_lines<false, kEmax, TENSOR>(p.pz, nc, tw, cols, cols, prod, true, true);
    fft_lines<true, kEmax, TENSOR>(p.pz, nc, tw, cols, cols, cols, true, true);
    for (int v = threadIdx.x; v < Z * TC; v += blockDim.x) {
      const int z = v / TC, c = v - z * TC;
      const long long i = (long long)z * Y + y0 + c;
      if (c < nc && PF_CHECK(kChkBufStore, i, glim) && PF_CHECK_SMEM(kChkSmem, t + z * rs + c, 8))
        gplane[i] = t[z * rs + c];
    }
  } else {
    fft_lines<false, kEmax, TENSOR>(p.pz, nc, tw, cols, cols, cols, true, true);
    const long long out_off = ((long long)f * g.nx + kx) * plane;
    float2* o = p.out + out_off;
    for (int v = threadIdx.x; v < Z * TC; v += blockDim.x) {
      const int z = v / TC, c = v - z * TC;
      const long long i = (long long)z * Y + y0 + c;
      if (c < nc && PF_CHECK(kChkOut, i, p.out_len - out_off) && PF_CHECK_SMEM(kChkSmem, t + z * rs + c, 8))
        o[i] = cscale(t[z * rs + c], p.scale);
    }
  }
}
#endif  // PF_GENERIC_KERNELS

// ---------------------------------------------------------------------------
// Pass 3: inverse x transform, LCC, running max / argmax
// ---------------------------------------------------------------------------
struct Pass3Params {
  Geometry g;
  AxisPlan px;
  const float2* __restrict__ twx;
  const float2* __restrict__ buf;
  int npairs;                  // pairs in this batch
  long long first_rot;         // rotation index of pair 0, rotation a (local to the scan)
  long long nrot;
  long long rot_offset;        // added to the stored rotation index
  const unsigned char* __restrict__ lcc_mask;
  float norm_factor;           // number of mask voxels
  float* __restrict__ lcc;     // running best (float32)
  int* __restrict__ rot;       // running argmax
  int ty;
  int fp64;                    // 1: variance and LCC in float64
  int tma = 0;                 // fast path: tiles by one TMA tensor copy (the tensor map is a kernel argument)
  int* err = nullptr;          // set to 1 when a tile copy's wait runs out
  // fast path with gridDim.z == P > 1: the batch's pairs split into P parts
  // of ceil(npairs / P) in order; blocks with blockIdx.z == k > 0 take part k,
  // starting from 0, and keep their best in these arrays at offset (k-1)*N
  // (merged into lcc / rot afterwards in part order, earlier parts winning ties)
  float* __restrict__ part_lcc = nullptr;
  int* __restrict__ part_rot = nullptr;
  // with PF_FLAG_ROT_MAX: per rotation of the uploaded set, the best LCC over
  // the voxels inside the lcc mask and the voxel holding it, as one key:
  // (order-preserving key of the LCC) << 32 | voxel index (0: none yet)
  unsigned long long* __restrict__ rotmax = nullptr;
  long long buf_len = 0;       // elements of buf, of rotmax (bounds checks)
  long long rotmax_len = 0;
};

// order-preserving key of a float: a larger float has a larger key, and every
// float's key is above 0 (which stands for "no value")
__device__ __forceinline__ unsigned int float_key(float f) {
  const unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// (LCC, voxel) key of one voxel's value; NaN never counts (key 0)
__device__ __forceinline__ unsigned long long lcc_voxel_key(float v, long long voxel) {
  return v == v ? ((unsigned long long)float_key(v) << 32) | (unsigned long long)(unsigned int)voxel : 0ull;
}

// Block-wide max of each thread's keys (ka, kb) -- the best (LCC, voxel) of
// rotations ra and ra + 1 over the voxels the thread holds -- merged into
// rotmax[ra], rotmax[ra + 1] by one atomicMax each.  Every thread of the
// block calls it; `s_red` holds 64 keys; the caller's next barrier makes
// `s_red` reusable.  `len`: entries of rotmax (bounds checks).
__device__ __forceinline__ void rotmax_block(unsigned long long* rotmax, long long len, long long ra, bool has_b,
                                             unsigned long long ka, unsigned long long kb,
                                             unsigned long long* s_red) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long oa = __shfl_xor_sync(0xffffffffu, ka, off);
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, kb, off);
    ka = oa > ka ? oa : ka;
    kb = ob > kb ? ob : kb;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    s_red[warp] = ka;
    s_red[32 + warp] = kb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    unsigned long long a = 0, b = 0;
    for (int w = 0; w < nw; ++w) {
      a = s_red[w] > a ? s_red[w] : a;
      b = s_red[32 + w] > b ? s_red[32 + w] : b;
    }
    if (a && PF_CHECK(kChkRotation, ra, len)) atomicMax(rotmax + ra, a);
    if (has_b && b && PF_CHECK(kChkRotation, ra + 1, len)) atomicMax(rotmax + ra + 1, b);
  }
}

struct GlobalRowsLoad {  // line = f*ty + r, idx = kx: buf[f][kx][z][y0 + r]
  const float2* base;
  int ty, y0, ny, nz, nx, z;
  long long lim;          // elements from base on (bounds checks)
  __device__ __forceinline__ float2 load(int line, int idx) const {
    const int f = line / ty, r = line - f * ty;
    const int y = y0 + r;
    const long long i = (((long long)f * nx + idx) * nz + z) * ny + y;
    return y < ny && PF_CHECK(kChkBufLoad, i, lim) ? base[i] : make_float2(0.f, 0.f);
  }
};

// local variance Nm*ave2 - ave^2 and gcc / sqrt(var), with the subtraction
// carried in float-float (exact products by FMA, two-sum of the difference)
__device__ __forceinline__ float lcc_value(float gcc, float ave, float ave2, float nm) {
  const float p1 = ave2 * nm;
  const float e1 = fmaf(ave2, nm, -p1);
  const float p2 = ave * ave;
  const float e2 = fmaf(ave, ave, -p2);
  const float s = p1 - p2;
  const float bb = s - p1;
  const float err = (p1 - (s - bb)) + (-p2 - bb);
  const float var = s + ((err + e1) - e2);
  // rsqrt keeps the IEEE cases of gcc / sqrt(var): var == 0 -> +-inf (NaN for
  // gcc == 0), var < 0 -> NaN
  return gcc * rsqrtf(var);
}

// The same in float64: the local variance Nm*ave2 - ave^2 and the division by
// its square root.  The result is a float, so 1/sqrt(var) is taken to well
// past float precision without float64 sqrt and divide: a float rsqrtf seed
// (relative error ~2^-23) and one Newton-Raphson step for 1/sqrt in float64,
// y1 = y0 (1 + (1 - var y0^2) / 2), whose relative error is about
// 1.5 (2^-23)^2 ~ 2^-45; gcc * y1 is then rounded to float once.  Variances
// outside the seed's normal float range, zero, negative or NaN take
// gcc / sqrt(var) in float64 (its IEEE cases: +-inf, NaN).
__device__ __forceinline__ float lcc_value64(float gcc, float ave, float ave2, float nm) {
  const double var = (double)ave2 * (double)nm - (double)ave * (double)ave;
  if (var > 1e-30 && var < 1e30) {
    const double y0 = (double)rsqrtf((float)var);
    const double r = fma(-var * y0, y0, 1.0);
    const double y1 = fma(0.5 * y0, r, y0);
    return (float)((double)gcc * y1);
  }
  return (float)((double)gcc / sqrt(var));
}

constexpr int kMaxVoxPerThread = 8;   // pass 3: voxels per thread (tile rows * nx <= 8 * 256)
// fast pass 3: most voxels a tile (rows * nx) may hold
#ifndef PF_PASS3_MAXVOX
#define PF_PASS3_MAXVOX 2048
#endif
constexpr int kMaxVoxPass3Fast = PF_PASS3_MAXVOX;
// fast pass 3: resident blocks per SM that its register allocation must allow
#ifndef PF_PASS3_MINB
#define PF_PASS3_MINB 2
#endif
constexpr int kPass3BlocksPerSm = PF_PASS3_MINB;
// most blocks one tile's pairs are split over (fast pass 3)
constexpr int kPass3MaxParts = 4;

#ifdef PF_GENERIC_KERNELS
template <bool TC>
__global__ void __launch_bounds__(kThreadsLine) k_pass3(const Pass3Params p) {
  extern __shared__ float2 sm[];
  __shared__ unsigned long long s_red[64];
  const Geometry& g = p.g;
  const int X = g.nx;
  float2* tw = sm;
  float2* fld = sm + X;                      // [3][ty][X + kPad]
  const int rs = X + kPad;
  for (int i = threadIdx.x; i < X; i += blockDim.x) tw[i] = p.twx[i];
  __syncthreads();   // the twiddle table is read before the first barrier of the transform

  const int z = blockIdx.x;
  const int y0 = blockIdx.y * p.ty;
  const int nvox = p.ty * X;
  const long long zoff = (long long)z * g.ny * X;

  float best[kMaxVoxPerThread];
  int brot[kMaxVoxPerThread];
  unsigned int inmask = 0;
#pragma unroll
  for (int k = 0; k < kMaxVoxPerThread; ++k) {
    const int v = threadIdx.x + k * blockDim.x;
    best[k] = 0.f;
    brot[k] = 0;
    if (v < nvox) {
      const int r = v / X, x = v - r * X;
      const int y = y0 + r;
      const long long gi = zoff + (long long)y * X + x;
      if (y < g.ny && PF_CHECK(kChkVoxel, gi, (long long)g.nz * g.ny * X)) {
        best[k] = p.lcc[gi];
        brot[k] = p.rot[gi];
        if (p.lcc_mask[gi]) inmask |= 1u << k;
      }
    }
  }

  const long long fstride = (long long)g.nx * g.nz * g.ny;
  for (int pair = 0; pair < p.npairs; ++pair) {
    GlobalRowsLoad src{p.buf + (long long)pair * 3 * fstride, p.ty, y0, g.ny, g.nz, g.nx, z,
                       p.buf_len - (long long)pair * 3 * fstride};
    SmemLines lines{fld, rs, 1};
    fft_lines<true, kEmax, TC>(p.px, 3 * p.ty, tw, src, lines, lines, false, true);
    __syncthreads();
    const long long ra = p.first_rot + 2LL * pair;
    const bool has_b = ra + 1 < p.nrot;
    unsigned long long ka = 0, kb = 0;
#pragma unroll
    for (int k = 0; k < kMaxVoxPerThread; ++k) {
      if (inmask & (1u << k)) {
        const int v = threadIdx.x + k * blockDim.x;
        const int r = v / X, x = v - r * X;
        const bool in = PF_CHECK_SMEM(kChkSmem, fld + (2 * p.ty + r) * rs + x, 8);
        const float2 f0 = in ? fld[(0 * p.ty + r) * rs + x] : make_float2(0.f, 0.f);
        const float2 f1 = in ? fld[(1 * p.ty + r) * rs + x] : make_float2(0.f, 0.f);
        const float2 f2 = in ? fld[(2 * p.ty + r) * rs + x] : make_float2(0.f, 0.f);
        float la, lb;
        if (p.fp64) {
          la = lcc_value64(f0.x, f0.y, f2.x, p.norm_factor);
          lb = lcc_value64(f1.x, f1.y, f2.y, p.norm_factor);
        } else {
          la = lcc_value(f0.x, f0.y, f2.x, p.norm_factor);
          lb = lcc_value(f1.x, f1.y, f2.y, p.norm_factor);
        }
        if (la > best[k]) { best[k] = la; brot[k] = (int)(p.rot_offset + ra); }
        if (has_b && lb > best[k]) { best[k] = lb; brot[k] = (int)(p.rot_offset + ra + 1); }
        if (p.rotmax) {
          const long long gi = zoff + (long long)(y0 + r) * X + x;
          const unsigned long long qa = lcc_voxel_key(la, gi), qb = lcc_voxel_key(lb, gi);
          ka = qa > ka ? qa : ka;
          kb = qb > kb ? qb : kb;
        }
      }
    }
    if (p.rotmax) rotmax_block(p.rotmax, p.rotmax_len, ra, has_b, ka, kb, s_red);
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < kMaxVoxPerThread; ++k) {
    const int v = threadIdx.x + k * blockDim.x;
    if (v < nvox) {
      const int r = v / X, x = v - r * X;
      const int y = y0 + r;
      const long long gi = zoff + (long long)y * X + x;
      if (y < g.ny && PF_CHECK(kChkVoxel, gi, (long long)g.nz * g.ny * X)) {
        p.lcc[gi] = best[k];
        p.rot[gi] = brot[k];
      }
    }
  }
}

#endif  // PF_GENERIC_KERNELS

// ---------------------------------------------------------------------------
// Target spectra: x transform of two real fields (target', target'^2)
// ---------------------------------------------------------------------------
struct FwdXParams {
  Geometry g;
  AxisPlan px;
  const float2* __restrict__ twx;
  const float* __restrict__ in0;   // real field 0
  const float* __restrict__ in1;   // real field 1 (may be null: zeros)
  int square1;                     // field 1 = in0^2 (in1 ignored)
  float2* __restrict__ buf;        // [2][kx][z][y]
  int ty;
  long long buf_len = 0;           // elements of buf (bounds checks)
};

#ifdef PF_GENERIC_KERNELS
__global__ void __launch_bounds__(kThreadsLine) k_fwd_x_real(const FwdXParams p) {
  extern __shared__ float2 sm[];
  const Geometry& g = p.g;
  const int X = g.nx;
  float2* tw = sm;
  float2* fld = sm + X;
  const int rs = X + kPad;
  for (int i = threadIdx.x; i < X; i += blockDim.x) tw[i] = p.twx[i];
  const int z = blockIdx.x;
  const int y0 = blockIdx.y * p.ty;
  for (int v = threadIdx.x; v < p.ty * X; v += blockDim.x) {
    const int r = v / X, x = v - r * X;
    const int y = y0 + r;
    float a = 0.f, b = 0.f;
    const long long gi = ((long long)z * g.ny + y) * X + x;
    if (y < g.ny && PF_CHECK(kChkVoxel, gi, (long long)g.nz * g.ny * X)) {
      a = p.in0[gi];
      b = p.square1 ? a * a : (p.in1 ? p.in1[gi] : 0.f);
    }
    if (PF_CHECK_SMEM(kChkSmem, fld + (p.ty + r) * rs + x, 8)) {
      fld[r * rs + x] = make_float2(a, 0.f);
      fld[(p.ty + r) * rs + x] = make_float2(b, 0.f);
    }
  }
  __syncthreads();
  SmemLines lines{fld, rs, 1};
  TransposedStore out{p.buf, p.ty, y0, g.ny, g.nz, g.nx, z, p.buf_len};
  fft_lines<false, kEmax>(p.px, 2 * p.ty, tw, lines, lines, out, true, false);
}

#endif  // PF_GENERIC_KERNELS

// ---------------------------------------------------------------------------
// Unit-level kernels mirroring the reference's native helpers
// ---------------------------------------------------------------------------
#ifdef PF_GENERIC_KERNELS
// rotate_grid3d (_extensions.c:7-196): writes out only inside the sphere
__global__ void k_rotate_grid(Geometry g, GatherSrc src, RotFixed R, const double* __restrict__ rd, int radius,
                              int nearest, double* __restrict__ out) {
  const long long n = (long long)g.nz * g.ny * g.nx;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % g.nx);
    const int y = (int)((i / g.nx) % g.ny);
    const int z = (int)(i / ((long long)g.nx * g.ny));
    // offsets in [-radius, radius] that land on this voxel; the last in loop order wins
    int cz = -1000000, cy = 0, cx = 0;
    bool found = false;
    for (int oz = z - 2 * g.nz; oz <= radius; oz += g.nz) {
      if (oz < -radius) continue;
      for (int oy = y - 2 * g.ny; oy <= radius; oy += g.ny) {
        if (oy < -radius) continue;
        for (int ox = x - 2 * g.nx; ox <= radius; ox += g.nx) {
          if (ox < -radius) continue;
          if (oz * oz + oy * oy + ox * ox <= radius * radius) { cz = oz; cy = oy; cx = ox; found = true; }
        }
      }
    }
    if (!found) continue;
    float t, m;
    gather_point(g, src, R, rd, cz, cy, cx, t, m);
    out[i] = nearest ? (double)m : (double)t;
  }
}

// conj_multiply (_powerfit.pyx:45-53), complex128
__global__ void k_conj_multiply(const double2* __restrict__ a, const double2* __restrict__ b, double2* __restrict__ o,
                                long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 x = a[i], y = b[i];
    o[i] = make_double2(__dadd_rn(__dmul_rn(x.x, y.x), __dmul_rn(x.y, y.y)),
                        __dsub_rn(__dmul_rn(x.x, y.y), __dmul_rn(x.y, y.x)));
  }
}

// calc_lcc (_powerfit.pyx:56-72), float64
__global__ void k_calc_lcc(const double* __restrict__ gcc, const double* __restrict__ ave,
                           const double* __restrict__ ave2, const unsigned char* __restrict__ mask,
                           double* __restrict__ lcc, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (mask[i]) {
      // separate rounding of the square and the difference, as the reference
      // computes it (no fused multiply-add): ave2 == ave^2 gives var == 0
      const double var = __dsub_rn(ave2[i], __dmul_rn(ave[i], ave[i]));
      lcc[i] = __ddiv_rn(gcc[i], __dsqrt_rn(var));
    }
  }
}

// PowerFitter._combine (powerfitter.py:146-163): strict > merge of rotation shards
__global__ void k_combine(const float* __restrict__ part_lcc, const int* __restrict__ part_rot, long long rot_add,
                          float* __restrict__ lcc, int* __restrict__ rot, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float v = part_lcc[i];
    if (v > lcc[i]) { lcc[i] = v; rot[i] = (int)(part_rot[i] + rot_add); }
  }
}

// merge of `nparts` part arrays (stride n) into lcc / rot, in part order:
// the same as k_combine once per part, so earlier parts keep their ties
__global__ void k_combine_parts(const float* __restrict__ part_lcc, const int* __restrict__ part_rot, int nparts,
                                float* __restrict__ lcc, int* __restrict__ rot, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float best = lcc[i];
    int r = 0;
    bool won = false;
    for (int k = 0; k < nparts; ++k) {
      const float v = part_lcc[k * n + i];
      if (v > best) { best = v; r = part_rot[k * n + i]; won = true; }
    }
    if (won) { lcc[i] = best; rot[i] = r; }
  }
}

#endif  // PF_GENERIC_KERNELS

}  // namespace pf
