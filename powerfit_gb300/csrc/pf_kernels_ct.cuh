// Fast-path kernels for grids whose edges are compile-time constants.
//
// Same three passes and buffer layout as pf_kernels.cuh, plus pruning of the
// (z, y) rows that the rotation cannot reach: with re = min(rmax, reff), a
// row whose offsets satisfy cz^2 + cy^2 > re^2 holds only zeros for every
// rotation, so pass 1 neither transforms nor stores it and pass 2 reads zeros
// for it without touching memory.
#pragma once
#include <cuda.h>   // CUtensorMap (the pass-3 tile copies)
#include <algorithm>
#include <cstring>
#include <cooperative_groups.h>
#include "pf_fft_ct.cuh"
#include "pf_kernels.cuh"

namespace pf {

__device__ __forceinline__ bool row_in_disk(const Geometry& g, int cz, int cy, int re2) {
  return cz * cz + cy * cy <= re2;
}

// ---------------------------------------------------------------------------
// Pass 1 (fast): gather + forward x transform of rows inside the disk
// ---------------------------------------------------------------------------
template <int X>
struct RowListStore {  // line = f*ty + c (row c of the chunk); idx = kx
  float2* base;
  const int4* rows;    // shared-memory copy of the chunk's row entries
  int ty, nr, ny, nz;
  long long lim;       // elements from base on (bounds checks)
  __device__ __forceinline__ void store(int line, int idx, float2 v) const {
    const int f = line / ty, c = line - f * ty;
    if (c < nr && PF_CHECK(kChkRowList, c, 32)) {
      const int4 e = rows[c];
      const long long i = (((long long)f * X + idx) * nz + e.x) * ny + e.y;
      if (PF_CHECK(kChkRowList, e.x, nz) & PF_CHECK(kChkRowList, e.y, ny) & PF_CHECK(kChkBufStore, i, lim)) base[i] = v;
    }
  }
};

// periodic index in [0, N) of any offset (a remainder by a compile-time N,
// no branches); rotations keep offsets within [-N, 2N), but any matrix the
// library accepts still lands inside the grid
template <int N>
__device__ __forceinline__ int wrap_ct(int i) {
  const int r = i % N;
  return r < 0 ? r + N : r;
}

// gather_point for an N^3 grid known at compile time, with the row part of q
// (the cz and cy terms) precomputed: q = qrow + cx * (r0, r1, r2).  The same
// values as gather_point, with 32-bit voxel indices, branch-free wrapping and
// the template read as x-neighbour pairs (one 8-byte load per trilinear edge).
template <int N>
__device__ __forceinline__ void gather_point_ct(const GatherSrc& src, const RotFixed& R, const double* __restrict__ rd,
                                                const long long* qrow, int cz, int cy, int cx, float& t, float& m) {
  const long long qx = qrow[0] + R.r[0] * cx;
  const long long qy = qrow[1] + R.r[1] * cx;
  const long long qz = qrow[2] + R.r[2] * cx;
  {
    const int x0 = (int)(qx >> 32), y0 = (int)(qy >> 32), z0 = (int)(qz >> 32);
    const float fx = frac_to_float((unsigned int)qx);
    const float fy = frac_to_float((unsigned int)qy);
    const float fz = frac_to_float((unsigned int)qz);
    const int ix0 = wrap_ct<N>(x0);
    const int iy0 = wrap_ct<N>(y0) * N, iy1 = wrap_ct<N>(y0 + 1) * N;
    const int iz0 = wrap_ct<N>(z0) * (N * N), iz1 = wrap_ct<N>(z0 + 1) * (N * N);
    if (!(PF_CHECK(kChkGather, ix0, N) & PF_CHECK(kChkGather, iy0, N * N) & PF_CHECK(kChkGather, iy1, N * N) &
          PF_CHECK(kChkGather, iz0, N * N * N) & PF_CHECK(kChkGather, iz1, N * N * N))) {
      t = m = 0.f;
      return;
    }
    const float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
    const float2* T = src.tmpl_pairs;
    const float2 a00 = __ldg(T + (iz0 + iy0 + ix0)), a10 = __ldg(T + (iz0 + iy1 + ix0));
    const float2 a01 = __ldg(T + (iz1 + iy0 + ix0)), a11 = __ldg(T + (iz1 + iy1 + ix0));
    const float c00 = a00.x * gx + a00.y * fx;
    const float c10 = a10.x * gx + a10.y * fx;
    const float c01 = a01.x * gx + a01.y * fx;
    const float c11 = a11.x * gx + a11.y * fx;
    const float c0 = c00 * gy + c10 * fy;
    const float c1 = c01 * gy + c11 * fy;
    t = c0 * gz + c1 * fz;
  }
  {
    const int x0 = round_fixed(qx, rd, 0, 3, 6, cz, cy, cx);
    const int y0 = round_fixed(qy, rd, 1, 4, 7, cz, cy, cx);
    const int z0 = round_fixed(qz, rd, 2, 5, 8, cz, cy, cx);
    const int i = wrap_ct<N>(z0) * (N * N) + wrap_ct<N>(y0) * N + wrap_ct<N>(x0);
    m = PF_CHECK(kChkGather, i, N * N * N) ? __ldg(src.mask + i) : 0.f;
  }
}

// Pass 1 over a list of the (z, y) rows the rotation can reach (built on the
// host from the template's support): every block transforms `ty` such rows,
// none is empty and none is outside the reach.
template <int X>
__global__ void PF_PASS1_BOUNDS k_pass1_ct(const Pass1Params p, const int re2) {
  extern __shared__ float2 sm[];
  const Geometry& g = p.g;
  constexpr int rs = X + kPad;
  float2* tw = sm;
  float2* fld = sm + X;
  __shared__ int4 s_row[32];
  __shared__ int s_start[33];
  if (!PF_CHECK(kChkRowList, p.ty - 1, 32)) return;     // tile rows beyond the row arrays (whole block)
  const int c0 = blockIdx.x * p.ty;
  const int nr = min(p.ty, p.nrows - c0);
  if (threadIdx.x < nr && PF_CHECK(kChkRowList, c0 + threadIdx.x, p.nrows)) s_row[threadIdx.x] = p.rows[c0 + threadIdx.x];
  for (int i = threadIdx.x; i < X; i += kThreadsLine) tw[i] = p.twx[i];
  for (int v = threadIdx.x; v < 3 * p.ty * rs; v += kThreadsLine)
    if (PF_CHECK_SMEM(kChkSmem, fld + v, 8)) fld[v] = make_float2(0.f, 0.f);
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int c = 0; c < p.ty; ++c) {
      s_start[c] = acc;
      if (c < nr) acc += s_row[c].z;
    }
    s_start[p.ty] = acc;
  }

  const int pair = blockIdx.z;
  const long long ra = p.first_rot + 2LL * pair, rb = ra + 1;
  const bool has_a = ra < p.nrot, has_b = rb < p.nrot;
  const RotFixed Ra = p.rots[has_a ? ra : 0];
  const RotFixed Rb = p.rots[has_b ? rb : 0];
  const double* rda = p.rotd + 9 * (has_a ? ra : 0);
  const double* rdb = p.rotd + 9 * (has_b ? rb : 0);
  // row part of q = R^T p for both rotations (cz and cy terms), one row per thread
  __shared__ long long s_q[32][2][3];
  if (threadIdx.x < nr) {
    const int4 e = s_row[threadIdx.x];
    const long long cz = signed_coord(e.x, g.nz), cy = signed_coord(e.y, g.ny);
    s_q[threadIdx.x][0][0] = Ra.r[6] * cz + Ra.r[3] * cy;
    s_q[threadIdx.x][0][1] = Ra.r[7] * cz + Ra.r[4] * cy;
    s_q[threadIdx.x][0][2] = Ra.r[8] * cz + Ra.r[5] * cy;
    s_q[threadIdx.x][1][0] = Rb.r[6] * cz + Rb.r[3] * cy;
    s_q[threadIdx.x][1][1] = Rb.r[7] * cz + Rb.r[4] * cy;
    s_q[threadIdx.x][1][2] = Rb.r[8] * cz + Rb.r[5] * cy;
  }
  __syncthreads();

  // gather the points inside the sphere, spread evenly over the threads
  const int total = s_start[p.ty];
  for (int k = threadIdx.x; k < total; k += kThreadsLine) {
    // row c of point k: the last row whose start is <= k (starts are
    // nondecreasing and every listed row holds points), by binary search
    int c = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1)
      if (c + step < p.ty && s_start[c + step] <= k) c += step;
    const int i = k - s_start[c];
    const int4 e = s_row[c];
    int x, cx;
    if (e.z == X) { x = i; cx = signed_coord(i, X); }
    else { cx = i - (e.z - 1) / 2; x = cx < 0 ? cx + X : cx; }
    const int cz = signed_coord(e.x, g.nz), cy = signed_coord(e.y, g.ny);
    float ta = 0.f, ma = 0.f, tb = 0.f, mb = 0.f;
    if (has_a) gather_point_ct<X>(p.src, Ra, rda, s_q[c][0], cz, cy, cx, ta, ma);
    if (has_b) gather_point_ct<X>(p.src, Rb, rdb, s_q[c][1], cz, cy, cx, tb, mb);
    if (PF_CHECK(kChkRowList, x, X) && PF_CHECK_SMEM(kChkSmem, fld + (2 * p.ty + c) * rs + x, 8)) {
      fld[(0 * p.ty + c) * rs + x] = make_float2(ta, -ma);
      fld[(1 * p.ty + c) * rs + x] = make_float2(tb, -mb);
      fld[(2 * p.ty + c) * rs + x] = make_float2(ma * ma, -(mb * mb));
    }
  }
  __syncthreads();
  SmemLines lines{fld, rs, 1};
  const long long pair_off = (long long)pair * 3 * X * g.nz * g.ny;
  RowListStore<X> out{p.buf + pair_off, s_row, p.ty, nr, g.ny, g.nz, p.buf_len - pair_off};
  ct_lines<X, false, kThreadsLine, kEmax>(3 * p.ty, tw, lines, lines, out, true, false);
}

// ---------------------------------------------------------------------------
// Pass 2 (fast): (z, y) plane per (pair, field, kx)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

struct GlobalRows {  // rows of a plane in global memory: line = z, idx = y
  float2* __restrict__ base;
  int ny;
  long long lim;      // elements from base on (bounds checks)
  __device__ __forceinline__ void store(int line, int idx, float2 v) const {
    const long long i = (long long)line * ny + idx;
    if (PF_CHECK(kChkBufStore, i, lim)) base[i] = v;
  }
};

struct SpectrumOperand {  // target spectrum plane [kz][ky] of this kx
  const float2* __restrict__ spec;
  int ny;
  long long lim;      // elements from spec on (bounds checks)
  __device__ __forceinline__ float2 fetch(int ky, int kz) const {
    const long long i = (long long)kz * ny + ky;
    return PF_CHECK(kChkSpectrum, i, lim) ? __ldg(spec + i) : make_float2(0.f, 0.f);
  }
};

// Columns of the plane for the first forward z stage: rows of the zero band
// (the z planes beyond the reach, zlo < z < hi) read as zeros without touching
// shared memory, so the copy-in never stores them.
struct BandCols {  // line = y (column), idx = z
  const float2* base;
  int rs, zlo, hi;
  __device__ __forceinline__ float2 load(int line, int idx) const {
    const float2* q = base + idx * rs + line;
    const bool in = idx <= zlo || idx >= hi;
    return (in && PF_CHECK_SMEM(kChkSmem, q, 8)) ? *q : make_float2(0.f, 0.f);
  }
};

// Rows of the valid z planes from valid row i0 on (line l -> valid row i0 + l)
struct RowMapLinesOff {
  float2* base;
  int rs, zlo, shift, i0;
  __device__ __forceinline__ int row(int l) const {
    const int i = i0 + l;
    return i <= zlo ? i : i + shift;
  }
  __device__ __forceinline__ float2 load(int line, int idx) const {
    const float2* q = base + row(line) * rs + idx;
    return PF_CHECK_SMEM(kChkSmem, q, 8) ? *q : make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ void store(int line, int idx, float2 v) const {
    float2* q = base + row(line) * rs + idx;
    if (PF_CHECK_SMEM(kChkSmem, q, 8)) *q = v;
  }
};

// Plane pass in teams: 1 (default) splits the block into teams of four warps
// where the plane is square and its lines split into 16 per team (64^2 and
// 128^2 planes); each team transforms its own 16 rows or columns and waits on
// its own barrier, with block barriers only where the transform direction
// changes (rows -> columns -> rows).  0: every stage block-wide.
#ifndef PF_P2_GROUPS
#define PF_P2_GROUPS 1
#endif

// Pass-2 copy-in: 1 (default) copies only the valid z rows and lets the first
// z stage read the zero band as zeros (BandCols); 0 stores zeros in the band.
#ifndef PF_P2_BAND
#define PF_P2_BAND 1
#endif

// Block shape of the plane pass: a plane of 128 x 128 or more fills one block
// per SM (shared memory), which then runs 1024 threads; smaller planes run two
// 512-thread blocks per SM, and planes of at most 32 x 32 (whose stages hold
// 128 to 256 butterflies) eight 128-thread blocks per SM, so that every
// thread has a butterfly.  All leave 64 registers a thread.
template <int Y, int Z>
struct PlaneLaunch {
  static constexpr bool kBig = Y * Z >= 128 * 128;
  static constexpr bool kSmall = Y * Z <= 32 * 32;
  static constexpr int kThreads = kBig ? 1024 : (kSmall ? 128 : 512);
  static constexpr int kMinBlocks = kBig ? 1 : (kSmall ? 8 : 2);
};

template <int Y, int Z>
__global__ void __launch_bounds__(PlaneLaunch<Y, Z>::kThreads, PlaneLaunch<Y, Z>::kMinBlocks)
    k_pass2_ct(const Pass2Params p, const int re2) {
  constexpr int kThreadsPlaneCt = PlaneLaunch<Y, Z>::kThreads;
  extern __shared__ float2 sm[];
  const Geometry& g = p.g;
  constexpr int rs = Y + kPad;
  float2* twy = sm;
  float2* twz = sm + Y;
  float2* pl = sm + Y + Z;
  float2* tly = pl + Z * rs;     // last inverse-y stage twiddles, [r][j]

  const int kx = blockIdx.x, f = blockIdx.y, pair = blockIdx.z;
  constexpr long long plane = (long long)Z * Y;
  const long long plane_off = (((long long)pair * p.nfield + f) * g.nx + kx) * plane;
  float2* gplane = p.buf + plane_off;
  const long long glim = p.buf_len - plane_off;
  const int nvz = g.nvz;
  const int lo_end = g.zlo, hi_start = Z - (nvz - g.zlo - 1);

  // copy-in: asynchronous 8-byte copies of the rows the rotation can reach,
  // zeros elsewhere (every thread keeps many copies in flight)
  const bool band = PF_P2_BAND && p.mode == 0;
  const int ncopy = band ? nvz * Y : Z * Y;    // band: the valid z rows only
  for (int v = threadIdx.x; v < ncopy; v += kThreadsPlaneCt) {
    const int i = v / Y, y = v - i * Y;
    const int z = (band && i > lo_end) ? i + (Z - nvz) : i;
    const bool valid = p.mode != 0 ||
                       ((z <= lo_end || z >= hi_start) && row_in_disk(g, signed_coord(z, Z), signed_coord(y, Y), re2));
    if (!PF_CHECK_SMEM(kChkSmem, pl + z * rs + y, 8)) continue;
    if (valid && PF_CHECK(kChkBufLoad, (long long)z * Y + y, glim)) cp_async8(pl + z * rs + y, gplane + (long long)z * Y + y);
    else pl[z * rs + y] = make_float2(0.f, 0.f);
  }
  for (int i = threadIdx.x; i < Y; i += kThreadsPlaneCt) twy[i] = p.twy[i];
  for (int i = threadIdx.x; i < Z; i += kThreadsPlaneCt) twz[i] = p.twz[i];
  ct_last_twiddles<Y, kThreadsPlaneCt>(p.twy, tly);
  cp_async_wait_all();
  __syncthreads();

  // teams of four warps owning 16 lines each (see PF_P2_GROUPS)
  constexpr int kTeam = 128, kLinesTeam = 16;
  constexpr bool kGroups = PF_P2_GROUPS && Y == Z && (Y / kLinesTeam) * kTeam == kThreadsPlaneCt;
  if constexpr (kGroups) {
    if (p.mode == 0) {
      using TM = GroupTeam<kTeam>;
      const int t = TM::team();
      const int l0 = kLinesTeam * t;
      // forward y: the team's valid rows l0 .. l0 + 15
      RowMapLinesOff vrows{pl, rs, g.zlo, Z - nvz, l0};
      ct_lines<Y, false, kTeam, kEmax, TM>(max(0, min(kLinesTeam, nvz - l0)), twy, vrows, vrows, vrows, true, true);
      __syncthreads();                       // every valid row transformed
      // z: the team's columns l0 .. l0 + 15 -- forward, product, inverse
      const long long spec_off = (long long)kx * plane + l0;
      const float2* spec = (f == p.nfield - 1 ? p.s2 : p.s1) + spec_off;
      SmemLines tcols{pl + l0, 1, rs};
      const SpectrumOperand op{spec, Y, p.spec_len - spec_off};
      if (band)
        ct_fwd_mul_inv<Z, kTeam, kEmax, TM>(kLinesTeam, twz, tcols, op, BandCols{pl + l0, rs, lo_end, hi_start}, true);
      else
        ct_fwd_mul_inv<Z, kTeam, kEmax, TM>(kLinesTeam, twz, tcols, op, tcols, true);
      __syncthreads();                       // every column transformed
      // inverse y: the team's rows l0 .. l0 + 15, the last stage straight to the buffer
      SmemLines trows{pl + l0 * rs, rs, 1};
      ct_head_inplace<Y, true, kTeam, kEmax, 0, TM>(kLinesTeam, twy, trows);
      ct_last_stage_out<Y, true, kTeam, TM>(kLinesTeam, tly, trows,
                                             GlobalRows{gplane + (long long)l0 * Y, Y, glim - (long long)l0 * Y});
      return;
    }
  }
  RowMapLines rows{pl, rs, g.zlo, Z - nvz};
  ct_lines<Y, false, kThreadsPlaneCt, kEmax>(nvz, twy, rows, rows, rows, true, true);
  SmemLines cols{pl, 1, rs};
  if (p.mode == 0) {
    const float2* spec = (f == p.nfield - 1 ? p.s2 : p.s1) + (long long)kx * plane;
    if (band)
      ct_fwd_mul_inv<Z, kThreadsPlaneCt, kEmax>(Y, twz, cols, SpectrumOperand{spec, Y, p.spec_len - (long long)kx * plane},
                                                BandCols{pl, rs, lo_end, hi_start}, true);
    else
      ct_fwd_mul_inv<Z, kThreadsPlaneCt, kEmax>(Y, twz, cols, SpectrumOperand{spec, Y, p.spec_len - (long long)kx * plane},
                                                cols, true);
    // inverse y: all stages but the last in place, the last one straight to the buffer
    SmemLines allrows{pl, rs, 1};
    ct_head_inplace<Y, true, kThreadsPlaneCt, kEmax, 0>(Z, twy, allrows);
    ct_last_stage_out<Y, true, kThreadsPlaneCt>(Z, tly, allrows, GlobalRows{gplane, Y, glim});
  } else {
    ct_lines<Z, false, kThreadsPlaneCt, kEmax>(Y, twz, cols, cols, cols, true, true);
    const long long out_off = ((long long)f * g.nx + kx) * plane;
    float2* o = p.out + out_off;
    for (int v = threadIdx.x; v < Z * Y; v += kThreadsPlaneCt) {
      const int z = v / Y, y = v - z * Y;
      if (PF_CHECK(kChkOut, (long long)z * Y + y, p.out_len - out_off) && PF_CHECK_SMEM(kChkSmem, pl + z * rs + y, 8))
        o[(long long)z * Y + y] = cscale(pl[z * rs + y], p.scale);
    }
  }
}

// ---------------------------------------------------------------------------
// Pass 2 (fast, clustered): the plane of one (pair, field, kx) shared by a
// cluster of CS blocks, for planes larger than one block's shared memory.
// Every exchange is a push: the last stage of a transform stores its outputs
// straight into the shared memory of the block that owns them next
// (st.shared::cluster), so no block ever waits on a remote load.
//
//   A. block c copies in its share of the valid z rows (rb = ceil(nvz / CS)
//      rows from valid row c*rb on) and y-transforms them; the last y stage
//      stores column ky into the column array of block ky / CW (CW = Y/CS);
//   B. block c z-transforms its CW columns, multiplies, inverse-z-transforms;
//      the last inverse stage stores row z into the row array of block z / ZB
//      (ZB = Z/CS);
//   C. block c inverse-y-transforms its ZB rows, the last stage straight to
//      the buffer in global memory.
//
// Cluster barriers (release / acquire) order the pushes: one before A's
// pushes (every block of the cluster is running), one after them, one after
// B's.  The row array holds A's input rows and C's rows: peers push into it
// only after the second barrier, when A is done with it.  After the third
// barrier no block touches another's memory, so every block may exit.
// ---------------------------------------------------------------------------
template <int CS>
struct ClusterBases {  // shared::cluster addresses of one array in each block of the cluster
  unsigned int a[CS];
  __device__ __forceinline__ unsigned int get(int r) const {
    unsigned int q = a[0];
#pragma unroll
    for (int k = 1; k < CS; ++k) q = (r == k) ? a[k] : q;
    return q;
  }
};

__device__ __forceinline__ unsigned int cluster_addr(const void* smem, int rank) {
  unsigned int d;
  const unsigned int a = (unsigned int)__cvta_generic_to_shared(smem);
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(rank));
  return d;
}

__device__ __forceinline__ void st_cluster(unsigned int addr, float2 v) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}

__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

template <int Y, int Z, int CS>
struct PushToColumns {  // A's last stage: line = own valid row, idx = ky -> column array of block ky / CW
  static constexpr int CW = Y / CS;
  ClusterBases<CS> cols;
  int i0, zlo, shift;
  __device__ __forceinline__ void store(int line, int ky, float2 v) const {
    const int i = i0 + line;
    const int z = i <= zlo ? i : i + shift;
    const int owner = ky / CW;
    const int off = z * (CW + kPad) + ky - owner * CW;    // column array [Z][CW + kPad] of the owner
    if (PF_CHECK(kChkCluster, owner, CS) & PF_CHECK(kChkCluster, off, Z * (CW + kPad)))
      st_cluster(cols.get(owner) + (unsigned int)(off * sizeof(float2)), v);
  }
};

template <int Y, int Z, int CS>
struct PushToRows {  // B's last stage: line = own column (ky - ky0), idx = z -> row array of block z / ZB
  static constexpr int ZB = Z / CS;
  ClusterBases<CS> rows;
  int ky0;
  int cap;             // elements of a block's row array (bounds checks)
  __device__ __forceinline__ void store(int line, int z, float2 v) const {
    const int owner = z / ZB;
    const int off = (z - owner * ZB) * (Y + kPad) + ky0 + line;
    if (PF_CHECK(kChkCluster, owner, CS) & PF_CHECK(kChkCluster, off, cap))
      st_cluster(rows.get(owner) + (unsigned int)(off * sizeof(float2)), v);
  }
};

template <int Y, int Z, int CS>
struct ClusterPlane {
  static constexpr int kCW = Y / CS;   // columns per block
  static constexpr int kZB = Z / CS;   // z rows per block after the z transform
  static_assert(Y % CS == 0 && Z % CS == 0, "cluster must divide the plane");
  // shared memory: twiddles (y, z, last-stage y table), column array [Z][CW + kPad],
  // row array [max(rb, ZB)][Y + kPad]
  static constexpr size_t smem(int nvz) {
    const int rb = (nvz + CS - 1) / CS;
    const int nr = rb > kZB ? rb : kZB;
    return ((size_t)2 * Y + Z + (size_t)Z * (kCW + kPad) + (size_t)nr * (Y + kPad)) * sizeof(float2);
  }
  // two 512-thread blocks per SM where two fit, else one of 1024 threads (64 registers either way)
  static constexpr bool kTwo = smem(Z) <= 113 * 1024;
  static constexpr int kThreads = kTwo ? 512 : 1024;
  static constexpr int kMinBlocks = kTwo ? 2 : 1;
};

template <int Y, int Z, int CS>
__global__ void __launch_bounds__(ClusterPlane<Y, Z, CS>::kThreads, ClusterPlane<Y, Z, CS>::kMinBlocks)
    k_pass2_cl(const Pass2Params p, const int re2) {
  namespace cg = cooperative_groups;
  constexpr int NT = ClusterPlane<Y, Z, CS>::kThreads;
  constexpr int CW = ClusterPlane<Y, Z, CS>::kCW, ZB = ClusterPlane<Y, Z, CS>::kZB;
  extern __shared__ float2 sm[];
  const int c = (int)cg::this_cluster().block_rank();
  cluster_arrive();                        // this block is running (waited on before the first push)
  const Geometry& g = p.g;
  const int nvz = g.nvz, zlo = g.zlo, shift = Z - nvz, hi_start = Z - (nvz - zlo - 1);
  const int rb = (nvz + CS - 1) / CS;
  float2* twy = sm;
  float2* twz = sm + Y;
  float2* tly = sm + Y + Z;                // last inverse-y stage twiddles, [r][j]
  float2* cols = sm + 2 * Y + Z;           // [Z][CW + kPad]
  float2* rows = cols + Z * (CW + kPad);   // A: [rb][Y + kPad] (own valid rows); C: [ZB][Y + kPad]

  const int kx = blockIdx.y, f = blockIdx.z % p.nfield, pair = blockIdx.z / p.nfield;
  constexpr long long plane = (long long)Z * Y;
  const long long plane_off = (((long long)pair * p.nfield + f) * g.nx + kx) * plane;
  float2* gplane = p.buf + plane_off;
  const long long glim = p.buf_len - plane_off;

  // A. own valid rows: the entries the rotation can reach, zeros elsewhere;
  // zeros in the column array's rows outside the valid planes (no block pushes those)
  const int i0 = c * rb;
  const int nown = max(0, min(rb, nvz - i0));
  for (int v = threadIdx.x; v < nown * Y; v += NT) {
    const int li = v / Y, y = v - li * Y;
    const int i = i0 + li;
    const int z = i <= zlo ? i : i + shift;
    if (!PF_CHECK_SMEM(kChkSmem, rows + li * (Y + kPad) + y, 8)) continue;
    if (row_in_disk(g, signed_coord(z, Z), signed_coord(y, Y), re2) && PF_CHECK(kChkBufLoad, (long long)z * Y + y, glim))
      cp_async8(rows + li * (Y + kPad) + y, gplane + (long long)z * Y + y);
    else
      rows[li * (Y + kPad) + y] = make_float2(0.f, 0.f);
  }
  for (int v = threadIdx.x; v < (hi_start - zlo - 1) * CW; v += NT) {
    const int zi = v / CW, col = v - zi * CW;
    if (PF_CHECK(kChkSmem, (zlo + 1 + zi) * (CW + kPad) + col, Z * (CW + kPad)))
      cols[(zlo + 1 + zi) * (CW + kPad) + col] = make_float2(0.f, 0.f);
  }
  for (int i = threadIdx.x; i < Y; i += NT) twy[i] = p.twy[i];
  for (int i = threadIdx.x; i < Z; i += NT) twz[i] = p.twz[i];
  ct_last_twiddles<Y, NT>(p.twy, tly);
  ClusterBases<CS> bcols, brows;
#pragma unroll
  for (int k = 0; k < CS; ++k) {
    bcols.a[k] = cluster_addr(cols, k);
    brows.a[k] = cluster_addr(rows, k);
  }
  cp_async_wait_all();
  __syncthreads();
  cluster_wait();                          // every block of the cluster is running
  SmemLines own_rows{rows, Y + kPad, 1};
  PushToColumns<Y, Z, CS> to_cols{bcols, i0, zlo, shift};
  ct_lines<Y, false, NT, kEmax>(nown, twy, own_rows, own_rows, to_cols, true, false);
  cluster_arrive();
  cluster_wait();                          // every column array is complete

  // B. own columns: z transform, product, inverse z; the last stage pushes rows
  SmemLines own_cols{cols, 1, CW + kPad};
  const long long spec_off = (long long)kx * plane + c * CW;
  const float2* spec = (f == p.nfield - 1 ? p.s2 : p.s1) + spec_off;
  PushToRows<Y, Z, CS> to_rows{brows, c * CW, max(rb, ZB) * (Y + kPad)};
  ct_fwd_mul_inv<Z, NT, kEmax>(CW, twz, own_cols, SpectrumOperand{spec, Y, p.spec_len - spec_off}, own_cols, true,
                               &to_rows);
  cluster_arrive();
  cluster_wait();                          // every row array is complete; no more remote stores

  // C. own z rows: inverse y, the last stage straight to the buffer
  SmemLines out_rows{rows, Y + kPad, 1};
  ct_head_inplace<Y, true, NT, kEmax, 0>(ZB, twy, out_rows);
  ct_last_stage_out<Y, true, NT>(ZB, tly, out_rows, GlobalRows{gplane + (long long)c * ZB * Y, Y,
                                                                glim - (long long)c * ZB * Y});
}

// Whether one block holds a whole N x N plane (twiddles, plane, last-stage
// twiddle table) within the 227 KB a block may use.
template <int N>
constexpr bool plane_fits_block() {
  return ((size_t)2 * N + (size_t)N * (N + kPad) + N) * sizeof(float2) <= 227 * 1024;
}

// Cluster size of the clustered plane pass per fast size (0: one block per
// plane).  Where one block's plane fits, one block per plane is faster: at
// 128^3 a two-block cluster ran pass 2 1.6x slower than one 1024-thread block,
// its distributed-shared-memory reads waiting on the load queue.  Larger
// planes (192^2: 296 KB) are shared by four blocks.
#ifndef PF_CLUSTER_PLANE
#define PF_CLUSTER_PLANE 0
#endif
template <int N>
struct ClusterOf {
  static constexpr int kCS = PF_CLUSTER_PLANE ? PF_CLUSTER_PLANE : (plane_fits_block<N>() ? 0 : 4);
};

// ---------------------------------------------------------------------------
// Pass 3 (fast): inverse x transform, LCC, running max / argmax
// ---------------------------------------------------------------------------

// Shared-memory bytes of pass 3 for `nbuf` tile buffers ([3][X][ty] complex).
// float2 slots holding the list of a tile's voxels inside the lcc mask (one 16-bit entry each)
__host__ __device__ inline int pass3_list_slots(int X, int ty) { return (ty * X * 2 + 7) / 8; }

// twiddles, the voxel list, nbuf tile buffers (on a 128-byte boundary: 128 bytes of slack)
__host__ __device__ inline size_t pass3_smem(int X, int ty, int nbuf) {
  return ((size_t)X + pass3_list_slots(X, ty) + (size_t)nbuf * 3 * ty * X) * sizeof(float2) + 128;
}

// Tile of pass 3 for pair `pair` by one TMA tensor copy: the buffer viewed as
// a 5-D tensor (y, z, kx, field, pair), box (ty, 1, X, 3, 1) at (y0, z, 0, 0,
// pair), lands in shared memory as [field][kx][row] -- the tile's layout --
// with rows beyond the grid filled with zeros; it completes on `bar`.
__device__ __forceinline__ void pass3_tile_tma(const CUtensorMap* map, float2* dst, unsigned long long* bar, int y0,
                                               int z, int pair, unsigned int bytes) {
  const unsigned int b = smem_u32(bar), d = smem_u32(dst);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
      "[%7];" ::"r"(d),
      "l"(map), "r"(y0), "r"(z), "r"(0), "r"(0), "r"(pair), "r"(b)
      : "memory");
}

// Bounded wait for completion `parity` of a tile barrier (2 s on the global timer).
__device__ __forceinline__ bool pass3_tile_wait(unsigned long long* bar, unsigned int parity) {
  const unsigned int b = smem_u32(bar);
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (;;) {
    unsigned int done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(b), "r"(parity)
        : "memory");
    if (done) return true;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > 2000000000ull) return false;
  }
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}

// The pass-3 tile keeps the global order: fld[f][kx][r] (r = row of the tile,
// fastest), so a run of `ty` rows of one (f, kx) is one contiguous copy.
// Lines of the x transform are (f, r): element kx of line f*ty + r sits at
// (f*X + kx)*ty + r, consecutive lines are consecutive words.
struct TileLines {
  float2* base;
  int sh, ty, xty;      // log2(ty), ty, X*ty
  __device__ __forceinline__ int off(int line) const { return (line >> sh) * xty + (line & (ty - 1)); }
  __device__ __forceinline__ float2 load(int line, int idx) const {
    const float2* q = base + off(line) + idx * ty;
    return PF_CHECK_SMEM(kChkSmem, q, 8) ? *q : make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ void store(int line, int idx, float2 v) const {
    float2* q = base + off(line) + idx * ty;
    if (PF_CHECK_SMEM(kChkSmem, q, 8)) *q = v;
  }
};

template <int X, int NT>
__device__ __forceinline__ void pass3_prefetch(const float2* __restrict__ base, long long lim, float2* fld, int ty,
                                               int y0, int ny, int nz, int z) {
  // buf[f][kx][z][y0 .. y0+ty) -> fld[(f*X + kx)*ty .. +ty): 16-byte copies (two rows each);
  // `lim`: elements from base on (bounds checks)
  const int halfty = ty >> 1;
  const int n = 3 * X * halfty;
  const int sh = __ffs(halfty) - 1;
  const long long zrow = (long long)z * ny + y0;
  if (y0 + ty <= ny) {
    for (int v = threadIdx.x; v < n; v += NT) {
      const int fk = v >> sh, part = v & (halfty - 1);
      const long long i = (long long)fk * nz * ny + zrow + 2 * part;
      if (PF_CHECK(kChkBufLoad, i + 1, lim) && PF_CHECK_SMEM(kChkSmem, fld + fk * ty + 2 * part, 16))
        cp_async16(fld + fk * ty + 2 * part, base + i);
    }
  } else {   // last tile of an edge not divisible by ty
    for (int v = threadIdx.x; v < 3 * X * ty; v += NT) {
      const int fk = v / ty, r = v - fk * ty;
      const long long i = (long long)fk * nz * ny + zrow + r;
      if (!PF_CHECK_SMEM(kChkSmem, fld + fk * ty + r, 8)) continue;
      if (y0 + r < ny && PF_CHECK(kChkBufLoad, i, lim)) cp_async8(fld + fk * ty + r, base + i);
      else fld[fk * ty + r] = make_float2(0.f, 0.f);
    }
  }
}

// Block shape of pass 3: NT threads, two blocks per SM, every voxel of a tile
// (at most kMaxVoxPerThread * kThreadsLine) owned by one of VPT slots of a thread
#ifndef PF_PASS3_THREADS
#define PF_PASS3_THREADS 256
#endif
#ifndef PF_PASS3_EMAX
#define PF_PASS3_EMAX 16
#endif
// 1: pass 3 instantiated with the tile rows 8 and 16 as compile-time constants
#ifndef PF_P3_CT_TY
#define PF_P3_CT_TY 1
#endif
constexpr int kThreadsPass3Ct = PF_PASS3_THREADS;
constexpr int kVoxPass3Ct = (kMaxVoxPass3Fast + kThreadsPass3Ct - 1) / kThreadsPass3Ct;

// TY > 0: the tile rows as a compile-time constant (the launcher picks this
// instantiation when p.ty == TY), so every tile index folds into constants;
// TY == 0 reads them from p.ty.
//
// Tiles arrive by one TMA tensor copy each (p.tma, the normal build) or by
// 16-byte cp.async copies (the bounds-checked build, whose checks cover every
// copy, and contexts without a tensor map).
template <int X, int TY>
__global__ void __launch_bounds__(kThreadsPass3Ct, kPass3BlocksPerSm)
    k_pass3_ct(const Pass3Params p, const __grid_constant__ CUtensorMap tmap) {
  constexpr int NT = kThreadsPass3Ct, VPT = kVoxPass3Ct;
  extern __shared__ float2 sm[];
  const Geometry& g = p.g;
  const int ty = TY > 0 ? TY : p.ty;        // a power of two >= 2 on this path
  float2* tw = sm;
  unsigned short* s_list = reinterpret_cast<unsigned short*>(sm + X);
  float2* fbuf0 = reinterpret_cast<float2*>(
      (reinterpret_cast<unsigned long long>(sm + X + pass3_list_slots(X, ty)) + 127ull) & ~127ull);
#ifdef PF_BOUNDS_CHECK
  const bool tma = false;
#else
  const bool tma = p.tma != 0;
#endif
  __shared__ unsigned long long s_bar[2];   // tile barriers of the two buffers (TMA)
  unsigned int phase = 0;                   // bit b: parity of buffer b's next completion
  const int sh = TY > 0 ? ct_log2(TY) : __ffs(ty) - 1;
  const int fbuf_stride = 3 * ty * X;

  const int z = blockIdx.x;
  const int y0 = blockIdx.y * ty;
  const int nvox = ty * X;
  const long long zoff = (long long)z * g.ny * X;
  const long long fstride = (long long)X * g.nz * g.ny;

  // pairs of this block: all, or part blockIdx.z of gridDim.z when the pairs are split over several blocks
  const int per = (p.npairs + (int)gridDim.z - 1) / (int)gridDim.z;
  const int pb = min(p.npairs, (int)blockIdx.z * per);
  const int pe = min(p.npairs, pb + per);

  const unsigned int tile_bytes = (unsigned int)(fbuf_stride * sizeof(float2));
  // start the first tile's copies before anything else
  if (tma) {
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar[0])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar[1])) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      if (pb < pe) pass3_tile_tma(&tmap, fbuf0, &s_bar[0], y0, z, pb, tile_bytes);
    }
  } else {
    if (pb < pe)
      pass3_prefetch<X, NT>(p.buf + (long long)pb * 3 * fstride, p.buf_len - (long long)pb * 3 * fstride, fbuf0, ty,
                            y0, g.ny, g.nz, z);
    cp_async_commit();
  }
  for (int i = threadIdx.x; i < X; i += NT) tw[i] = p.twx[i];

  // voxel v of the tile: row r = v & (ty-1), column x = v >> log2(ty).  The
  // voxels inside the lcc mask (the only ones whose best value can change)
  // are listed in order; thread t keeps the running best of list entries
  // m = t + k NT in registers.
  unsigned int inmask = 0;
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    const int v = threadIdx.x + k * NT;
    if (v < nvox) {
      const int y = y0 + (v & (ty - 1));
      const long long gi = zoff + (long long)y * X + (v >> sh);
      if (y < g.ny && PF_CHECK(kChkVoxel, gi, (long long)g.nz * g.ny * X) && p.lcc_mask[gi]) inmask |= 1u << k;
    }
  }
  __shared__ int s_warp[NT / 32 + 1];
  __shared__ unsigned long long s_red[64];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int cnt = __popc(inmask);
  int incl = cnt;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int w = 0; w < NT / 32; ++w) {
      const int t = s_warp[w];
      s_warp[w] = acc;
      acc += t;
    }
    s_warp[NT / 32] = acc;
  }
  __syncthreads();
  {
    int pos = s_warp[warp] + incl - cnt;
#pragma unroll
    for (int k = 0; k < VPT; ++k)
      if (inmask & (1u << k)) {
        if (PF_CHECK(kChkVoxelList, pos, 4 * pass3_list_slots(X, ty))) s_list[pos] = (unsigned short)(threadIdx.x + k * NT);
        ++pos;
      }
  }
  __syncthreads();
  const int total = s_warp[NT / 32];
  const long long part_off = blockIdx.z == 0 ? 0 : (long long)(blockIdx.z - 1) * g.nz * g.ny * X;
  float* __restrict__ out_lcc = blockIdx.z == 0 ? p.lcc : p.part_lcc + part_off;
  int* __restrict__ out_rot = blockIdx.z == 0 ? p.rot : p.part_rot + part_off;
  float best[VPT];
  int brot[VPT];
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    const int m = threadIdx.x + k * NT;
    best[k] = 0.f;
    brot[k] = 0;
    if (m < total && blockIdx.z == 0 && PF_CHECK(kChkVoxelList, m, 4 * pass3_list_slots(X, ty))) {
      const int v = s_list[m];
      const long long gi = zoff + (long long)(y0 + (v & (ty - 1))) * X + (v >> sh);
      if (PF_CHECK(kChkVoxel, gi, (long long)g.nz * g.ny * X)) {
        best[k] = p.lcc[gi];
        brot[k] = p.rot[gi];
      }
    }
  }

  for (int pair = pb; pair < pe; ++pair) {
    const int b = (pair - pb) & 1;
    float2* fld = fbuf0 + b * fbuf_stride;
    if (tma) {
      // the other buffer was last read before the barrier that ended the previous pair
      if (pair + 1 < pe && threadIdx.x == 0)
        pass3_tile_tma(&tmap, fbuf0 + (b ^ 1) * fbuf_stride, &s_bar[b ^ 1], y0, z, pair + 1, tile_bytes);
      const bool ok = pass3_tile_wait(&s_bar[b], (phase >> b) & 1u);
      phase ^= 1u << b;
      if (__syncthreads_or(!ok)) {             // a tile did not arrive: record it, wait for the copy in flight, stop
        if (threadIdx.x == 0) {
          if (p.err) atomicExch(p.err, 1);
          if (pair + 1 < pe) pass3_tile_wait(&s_bar[b ^ 1], (phase >> (b ^ 1)) & 1u);
        }
        break;
      }
    } else {
      if (pair + 1 < pe) {
        pass3_prefetch<X, NT>(p.buf + (long long)(pair + 1) * 3 * fstride,
                              p.buf_len - (long long)(pair + 1) * 3 * fstride, fbuf0 + (b ^ 1) * fbuf_stride, ty, y0,
                              g.ny, g.nz, z);
        cp_async_commit();
        cp_async_wait_group<1>();
      } else {
        cp_async_wait_group<0>();
      }
      __syncthreads();
    }
    TileLines lines{fld, sh, ty, X * ty};
    ct_lines<X, true, NT, PF_PASS3_EMAX>(3 * ty, tw, lines, lines, lines, true, true);
    const long long ra = p.first_rot + 2LL * pair;
    const bool has_b = ra + 1 < p.nrot;
    unsigned long long ka = 0, kb = 0;
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
      const int m = threadIdx.x + k * NT;
      if (m < total && PF_CHECK(kChkVoxelList, m, 4 * pass3_list_slots(X, ty))) {
        const int v = s_list[m];
        const int r = v & (ty - 1), x = v >> sh;
        const int o = x * ty + r;
        const bool in = PF_CHECK(kChkVoxelList, v, nvox) && PF_CHECK_SMEM(kChkSmem, fld + 2 * X * ty + o, 8);
        const float2 f0 = in ? fld[o] : make_float2(0.f, 0.f);
        const float2 f1 = in ? fld[X * ty + o] : make_float2(0.f, 0.f);
        const float2 f2 = in ? fld[2 * X * ty + o] : make_float2(0.f, 0.f);
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
    // this tile buffer's generic reads and writes come before the next TMA copy into it
    if (tma) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    const int m = threadIdx.x + k * NT;
    if (m < total && PF_CHECK(kChkVoxelList, m, 4 * pass3_list_slots(X, ty))) {
      const int v = s_list[m];
      const long long gi = zoff + (long long)(y0 + (v & (ty - 1))) * X + (v >> sh);
      if (PF_CHECK(kChkVoxel, gi, (long long)g.nz * g.ny * X)) {
        out_lcc[gi] = best[k];
        out_rot[gi] = brot[k];
      }
    }
  }
}

// Launchers instantiated once per fast size (pf_fast_<n>.cu)
struct FastLaunch {
  void (*pass1)(const Pass1Params&, int re2, dim3 grid, size_t smem, cudaStream_t s);
  void (*pass2)(const Pass2Params&, int re2, dim3 grid, size_t smem, cudaStream_t s);
  void (*pass3)(const Pass3Params&, const CUtensorMap* map, dim3 grid, size_t smem, cudaStream_t s);
  cudaError_t (*set_attrs)(size_t smem_line, size_t smem_plane);
  bool cluster_plane;   // pass 2 (correlation) runs even where a plane exceeds one block's shared memory
};

template <int N>
struct FastSize {
  static void pass1(const Pass1Params& p, int re2, dim3 grid, size_t smem, cudaStream_t s) {
    k_pass1_ct<N><<<grid, kThreadsLine, smem, s>>>(p, re2);
  }
  // grid: (nx, fields, pairs) planes
  static void pass2(const Pass2Params& p, int re2, dim3 grid, size_t smem, cudaStream_t s) {
    constexpr int CS = ClusterOf<N>::kCS;
    if constexpr (CS > 0) {
      if (p.mode == 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CS, grid.x, grid.y * grid.z);
        cfg.blockDim = dim3(ClusterPlane<N, N, CS>::kThreads);
        cfg.dynamicSmemBytes = ClusterPlane<N, N, CS>::smem(p.g.nvz);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = CS;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, k_pass2_cl<N, N, CS>, p, re2);   // errors surface in cudaGetLastError
        return;
      }
    }
    // (planes beyond one block take the split path for the target spectra)
    if constexpr (plane_fits_block<N>()) k_pass2_ct<N, N><<<grid, PlaneLaunch<N, N>::kThreads, smem, s>>>(p, re2);
  }

  // compile-time tile rows where a tile of that many rows fits the block
  static constexpr bool kTy16 = PF_P3_CT_TY && 16 * N <= kMaxVoxPass3Fast;
  static constexpr bool kTy8 = PF_P3_CT_TY && 8 * N <= kMaxVoxPass3Fast;
  // `map`: the tensor map of the tiles (p.tma set), or null (cp.async copies)
  static void pass3(const Pass3Params& p, const CUtensorMap* map, dim3 grid, size_t smem, cudaStream_t s) {
    CUtensorMap none;
    if (!map) std::memset(&none, 0, sizeof(none));
    const CUtensorMap& m = map ? *map : none;
    if constexpr (kTy16) {
      if (p.ty == 16) { k_pass3_ct<N, 16><<<grid, kThreadsPass3Ct, smem, s>>>(p, m); return; }
    }
    if constexpr (kTy8) {
      if (p.ty == 8) { k_pass3_ct<N, 8><<<grid, kThreadsPass3Ct, smem, s>>>(p, m); return; }
    }
    k_pass3_ct<N, 0><<<grid, kThreadsPass3Ct, smem, s>>>(p, m);
  }
  template <class K>
  static cudaError_t allow_smem(K kernel, size_t bytes) {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, kernel);
    if (e != cudaSuccess) return e;
    const size_t dyn = bytes > a.sharedSizeBytes ? bytes - a.sharedSizeBytes : 0;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  }
  // `smem_line` / `smem_plane`: total shared memory (static + dynamic) each kernel may use
  static cudaError_t set_attrs(size_t smem_line, size_t smem_plane) {
    cudaError_t e = allow_smem(k_pass1_ct<N>, smem_line);
    if (e == cudaSuccess) e = allow_smem(k_pass3_ct<N, 0>, smem_line);
    if constexpr (kTy16) {
      if (e == cudaSuccess) e = allow_smem(k_pass3_ct<N, 16>, smem_line);
    }
    if constexpr (kTy8) {
      if (e == cudaSuccess) e = allow_smem(k_pass3_ct<N, 8>, smem_line);
    }
    if constexpr (plane_fits_block<N>()) {
      if (e == cudaSuccess) e = allow_smem(k_pass2_ct<N, N>, smem_plane);
    }

    constexpr int CS = ClusterOf<N>::kCS;
    if constexpr (CS > 0) {
      if (e == cudaSuccess) e = allow_smem(k_pass2_cl<N, N, CS>, ClusterPlane<N, N, CS>::smem(N));
    }
    return e;
  }
  static FastLaunch table() { return FastLaunch{&pass1, &pass2, &pass3, &set_attrs, ClusterOf<N>::kCS > 0}; }
};

}  // namespace pf
