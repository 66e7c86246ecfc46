// C ABI of the GB300 LCC search: context, device memory, launches.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <mutex>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/powerfit_gb300.h"
#define PF_GENERIC_KERNELS 1  // the runtime-planned kernels are compiled in this unit only
#include "pf_kernels_ct.cuh"

using namespace pf;

// fast-path kernel tables, one translation unit per cubic grid size
pf::FastLaunch pf_fast_table_32();
pf::FastLaunch pf_fast_table_48();
pf::FastLaunch pf_fast_table_64();
pf::FastLaunch pf_fast_table_96();
pf::FastLaunch pf_fast_table_128();
pf::FastLaunch pf_fast_table_160();
pf::FastLaunch pf_fast_table_192();

namespace {

thread_local char g_err[512] = "";

void set_global_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

// Factor n into Stockham radices: fewest stages, then the largest smallest radix.
bool make_plan(int n, AxisPlan* pl) {
  static const int radices[] = {16, 12, 10, 8, 7, 6, 5, 4, 3, 2};
  std::vector<int> best, cur;
  int best_min = 0;
  auto consider = [&]() {
    int mn = *std::min_element(cur.begin(), cur.end());
    if (best.empty() || cur.size() < best.size() || (cur.size() == best.size() && mn > best_min)) {
      best = cur;
      best_min = mn;
    }
  };
  std::function<void(int, int)> rec = [&](int rem, int maxr) {
    if (rem == 1) {
      if (!cur.empty()) consider();
      return;
    }
    if (!best.empty() && cur.size() + 1 > best.size()) return;
    for (int r : radices) {
      if (r > maxr || rem % r) continue;
      cur.push_back(r);
      rec(rem / r, r);
      cur.pop_back();
    }
  };
  if (n == 1) {
    pl->n = 1;
    pl->nst = 1;
    pl->radix[0] = 1;
    return true;
  }
  rec(n, 16);
  if (best.empty() || (int)best.size() > kMaxStages) return false;
  pl->n = n;
  pl->nst = (int)best.size();
  for (int i = 0; i < pl->nst; ++i) pl->radix[i] = best[i];
  return true;
}

std::vector<float2> twiddles(int n) {
  std::vector<float2> t(n);
  for (int m = 0; m < n; ++m) {
    const double a = 2.0 * M_PI * (double)m / (double)n;
    t[m] = make_float2((float)std::cos(a), (float)-std::sin(a));
  }
  return t;
}

RotFixed to_fixed(const double* r) {
  RotFixed f;
  for (int i = 0; i < 9; ++i) f.r[i] = (long long)std::llround(r[i] * 4294967296.0);
  return f;
}

size_t line_smem(int X, int nf, int ty) { return ((size_t)X + (size_t)nf * ty * (X + kPad)) * sizeof(float2); }
// twiddles (y, z), the plane [Z][Y + kPad], the last inverse-y stage's twiddle table (Y)
size_t plane_smem(int Y, int Z) { return ((size_t)Y + Z + (size_t)Z * (Y + kPad) + Y) * sizeof(float2); }

}  // namespace

struct pf_ctx {
  int device = 0;
  int nz = 0, ny = 0, nx = 0;
  long long N = 0;
  cudaStream_t stream = nullptr;     // stream every launch and copy goes to
  cudaStream_t own_stream = nullptr; // the context's own stream (destroyed with it)
  AxisPlan px{}, py{}, pz{};
  float2 *twx = nullptr, *twy = nullptr, *twz = nullptr;
  float *tmpl = nullptr, *mask = nullptr;
  float2* tmpl_pairs = nullptr;      // fast pass 1: template as x-neighbour pairs
  unsigned char* lcc_mask = nullptr;
  float2* spec = nullptr;          // [2][kx][kz][ky]
  float* lcc = nullptr;
  int* rot = nullptr;
  float* part_lcc = nullptr;        // fast pass 3 split over several blocks per tile: best of the later parts
  int* part_rot = nullptr;
  int part_cap = 0;                  // part arrays of N voxels held in part_lcc / part_rot
  unsigned long long* rotmax = nullptr;   // PF_FLAG_ROT_MAX: per-rotation (best LCC, voxel) keys
  long long rotmax_cap = 0;
  float2* buf = nullptr;
  long long buf_pairs = 0;
  long long debug_buf_extent = -1;   // pf_debug_buffer_extent: extent of buf the kernels are told (-1: all)
  RotFixed* rots = nullptr;
  double* rotd = nullptr;
  int4* rows_reach = nullptr;       // fast pass 1: rows inside the reach disk (pruned)
  int4* rows_full = nullptr;        // fast pass 1: rows inside the rmax disk (no pruning)
  int nrows_reach = 0, nrows_full = 0;
  long long nrot = 0, rot_cap = 0;
  Geometry g{};
  int rmax = 0, reff_data = 0;
  float norm_factor = 0.f;
  bool have_target = false, have_template = false;
  int pairs = 1, ty1 = 16, ty3 = 16;
  size_t max_smem = 0;
  int num_sms = 0;
  bool fast = false;                 // compile-time-specialised kernels for this grid
  bool split = false;                // (z, y) plane larger than shared memory: pass 2 in three steps
  FastLaunch fl{};
  bool profiling = false;
  double ms[3] = {0, 0, 0};
  long long launches[3] = {0, 0, 0};
  std::vector<cudaEvent_t> ev_pool;
  struct Pending {
    int which, kernels;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;      // profiled launches whose events are not read yet
  CUtensorMap tmap3{};               // fast pass 3: the tiles of buf as a 5-D tensor (TMA copies)
  float2* tmap3_buf = nullptr;       // the buffer, pairs and tile rows the map was encoded for
  long long tmap3_pairs = 0;
  int tmap3_ty = 0;
  bool tmap3_ok = false;
  int* d_err = nullptr;              // device word: a tile copy's wait ran out (read by the synchronising calls)
  char err[512] = "";
};

namespace {

int fail(pf_ctx* c, int code, const char* fmt, ...) {
  char tmp[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(tmp, sizeof(tmp), fmt, ap);
  va_end(ap);
  if (c) snprintf(c->err, sizeof(c->err), "%s", tmp);
  snprintf(g_err, sizeof(g_err), "%s", tmp);
  return code;
}

#define PF_CUDA(c, call)                                                                            \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return fail((c), PF_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                       __FILE__, __LINE__);                                         \
  } while (0)

// Allocation-failure injection (tests of the error paths): the n-th device
// allocation from now on fails as if the device were out of memory (-1: never).
std::atomic<long long> g_fail_alloc_after{-1};

#ifdef PF_BOUNDS_CHECK
// readers of the bounds-check words of every translation unit (pf_check.cuh)
using CheckTake = int (*)(unsigned long long*, unsigned long long*);
std::vector<CheckTake>& check_units() {
  static std::vector<CheckTake> units;
  return units;
}
std::mutex& check_mutex() {
  static std::mutex m;
  return m;
}
#endif

int alloc(pf_ctx* c, void** p, size_t bytes) {
  long long k = g_fail_alloc_after.load();
  while (k >= 0 && !g_fail_alloc_after.compare_exchange_weak(k, k - 1)) {
  }
  if (k == 0) {
    *p = nullptr;
    return fail(c, PF_E_NOMEM, "cudaMalloc of %zu bytes failed: injected allocation failure", bytes);
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(c, PF_E_NOMEM, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
  }
  return PF_OK;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

// most voxels a pass-3 tile may hold on this context's path
long long max_vox3(const pf_ctx* c) {
  return c->fast ? (long long)kMaxVoxPass3Fast : (long long)kMaxVoxPerThread * kThreadsLine;
}

void choose_tiles(pf_ctx* c) {
  const int X = c->nx;
  int ty = 16;
  while (ty > 1 && ((long long)ty * X > (long long)kMaxVoxPerThread * kThreadsLine || line_smem(X, 3, ty) > 96 * 1024)) ty--;
  c->ty1 = ty;
  // pass 3: every voxel of a tile owned by one thread slot; enough tiles to
  // fill the machine (>= 4 per SM on 152 SMs)
  // a power of two (>= 2 on the fast path, whose pass 3 copies two rows per 16 bytes)
  const int ty3_min = c->fast ? 2 : 1;
  int ty3 = 16;
  while (ty3 > ty3_min && (long long)ty3 * X > max_vox3(c)) ty3 /= 2;
  while (ty3 > ty3_min && (long long)c->nz * ((c->ny + ty3 - 1) / ty3) < 4 * 152) ty3 /= 2;
  c->ty3 = ty3;
  // pairs per batch: intermediate spectra of one batch <= 64 MiB (L2-sized), at least 1, at most 16
  const long long per_pair = 3LL * c->N * (long long)sizeof(float2);
  long long p = (64LL << 20) / per_pair;
  c->pairs = (int)std::max(1LL, std::min(16LL, p));
}

// best of the later parts of a batch's pairs (fast pass 3 split over several
// blocks per tile): kPass3MaxParts - 1 arrays of N voxels, allocated at the
// first split (so that no later scan allocates, or waits, again); zero
// outside the lcc mask, which no block writes
int ensure_part(pf_ctx* c, int nparts) {
  if (c->part_cap >= nparts) return PF_OK;
  if (c->part_lcc) return fail(c, PF_E_ARG, "pass 3: %d part arrays asked, %d held", nparts, c->part_cap);
  const int cap = kPass3MaxParts - 1;
  const size_t n = (size_t)cap * c->N;
  int rc = alloc(c, (void**)&c->part_lcc, n * sizeof(float));
  if (!rc) rc = alloc(c, (void**)&c->part_rot, n * sizeof(int));
  if (rc) return rc;
  PF_CUDA(c, cudaMemsetAsync(c->part_lcc, 0, n * sizeof(float), c->stream));
  PF_CUDA(c, cudaMemsetAsync(c->part_rot, 0, n * sizeof(int), c->stream));
  c->part_cap = cap;
  return PF_OK;
}

// elements of buf the kernels may address (their bounds checks use it)
long long buf_extent(const pf_ctx* c) {
  const long long n = c->buf ? c->buf_pairs * 3 * c->N : 0;
  return c->debug_buf_extent >= 0 && c->debug_buf_extent < n ? c->debug_buf_extent : n;
}

// 1 (default): pass-3 tiles by TMA tensor copies where a tensor map can
// describe them; 0: always cp.async
#ifndef PF_P3_TMA
#define PF_P3_TMA 1
#endif

// cuTensorMapEncodeTiled from the driver (through the runtime: no link to
// the driver library), or null where it is not available
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)ptr;
  });
  return fn;
}

// The tensor map of the pass-3 tiles for tile rows `ty`: buf as (y, z, kx,
// field, pair) complex64 elements (8-byte words), box (ty, 1, nx, 3, 1);
// encoded again when the buffer, its pairs or the tile rows change.  False
// where TMA cannot take the tiles (edges beyond a box, row strides that are
// not multiples of 16 bytes, a shrunk buffer extent): pass 3 then copies
// with cp.async.
bool ensure_tile_map(pf_ctx* c, int ty) {
  if (c->tmap3_ok && c->tmap3_buf == c->buf && c->tmap3_pairs == c->buf_pairs && c->tmap3_ty == ty) return true;
  c->tmap3_ok = false;
  EncodeTiledFn fn = encode_tiled();
  if (!fn || !c->buf || c->nx > 256 || ty > 256 || ty < 2 || (c->ny * sizeof(float2)) % 16 ||
      (ty * sizeof(float2)) % 16 || c->debug_buf_extent >= 0)
    return false;
  const cuuint64_t e = sizeof(float2);
  const cuuint64_t dims[5] = {(cuuint64_t)c->ny, (cuuint64_t)c->nz, (cuuint64_t)c->nx, 3, (cuuint64_t)c->buf_pairs};
  const cuuint64_t strides[4] = {c->ny * e, (cuuint64_t)c->nz * c->ny * e, (cuuint64_t)c->nx * c->nz * c->ny * e,
                                 3ull * c->nx * c->nz * c->ny * e};
  const cuuint32_t box[5] = {(cuuint32_t)ty, 1, (cuuint32_t)c->nx, 3, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  if (fn(&c->tmap3, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 5, c->buf, dims, strides, box, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  c->tmap3_buf = c->buf;
  c->tmap3_pairs = c->buf_pairs;
  c->tmap3_ty = ty;
  c->tmap3_ok = true;
  return true;
}

// a tile copy of pass 3 whose wait ran out since the last check (clears the word)
int check_tile_error(pf_ctx* c) {
  if (!c->d_err) return PF_OK;
  int e = 0;
  PF_CUDA(c, cudaMemcpyAsync(&e, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  PF_CUDA(c, cudaStreamSynchronize(c->stream));
  if (e) {
    PF_CUDA(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
    return fail(c, PF_E_CUDA, "a pass-3 tile copy did not complete within its time limit");
  }
  return PF_OK;
}

int ensure_buf(pf_ctx* c, int pairs) {
  if (c->buf && c->buf_pairs >= pairs) return PF_OK;
  if (c->buf) cudaFree(c->buf);
  c->buf = nullptr;
  c->buf_pairs = 0;
  int rc = alloc(c, (void**)&c->buf, (size_t)pairs * 3 * c->N * sizeof(float2));
  if (rc) return rc;
  c->buf_pairs = pairs;
  return PF_OK;
}

void compute_geometry(pf_ctx* c, int reff) {
  Geometry& g = c->g;
  g.nz = c->nz;
  g.ny = c->ny;
  g.nx = c->nx;
  g.rmax = c->rmax;
  g.reff = reff;
  const int re = std::min(c->rmax, reff);
  if (2 * re + 1 >= c->nz) {
    g.nvz = c->nz;
    g.zlo = c->nz - 1;
  } else {
    g.nvz = 2 * re + 1;
    g.zlo = re;
  }
}

cudaEvent_t get_event(pf_ctx* c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

void collect_events(pf_ctx* c) {
  for (auto& pe : c->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, pe.a, pe.b) == cudaSuccess) {
      c->ms[pe.which] += ms;
      c->launches[pe.which] += pe.kernels;
    }
    c->ev_pool.push_back(pe.a);
    c->ev_pool.push_back(pe.b);
  }
  c->pending.clear();
}

// `launch()` issues the kernels of one pass and returns how many it launched
template <class Launch>
int timed_launch(pf_ctx* c, int which, Launch&& launch) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (c->profiling) {
    a = get_event(c);
    b = get_event(c);
    cudaEventRecord(a, c->stream);
  }
  const int kernels = launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(c, PF_E_CUDA, "kernel launch (pass %d) failed: %s", which + 1, cudaGetErrorString(e));
  if (c->profiling) {
    cudaEventRecord(b, c->stream);
    c->pending.push_back({which, kernels, a, b});
  }
  return PF_OK;
}

template <class K>
cudaError_t allow_smem(K kernel, size_t total) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kernel);
  if (e != cudaSuccess) return e;
  const size_t dyn = total > a.sharedSizeBytes ? total - a.sharedSizeBytes : 0;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
}

int set_smem_limits(pf_ctx* c) {
  // allow every kernel the device's opt-in maximum (static + dynamic); a
  // launch only takes what it asks for
  const size_t m = c->max_smem;
  PF_CUDA(c, allow_smem(k_pass1<false>, m));
  PF_CUDA(c, allow_smem(k_pass3<false>, m));
  PF_CUDA(c, allow_smem(k_fwd_x_real, m));
  PF_CUDA(c, allow_smem(k_pass2<false>, m));
  PF_CUDA(c, allow_smem(k_split_rows<false>, m));
  PF_CUDA(c, allow_smem(k_split_cols<false>, m));
  PF_CUDA(c, allow_smem(k_pass1<true>, m));
  PF_CUDA(c, allow_smem(k_pass3<true>, m));
  PF_CUDA(c, allow_smem(k_pass2<true>, m));
  PF_CUDA(c, allow_smem(k_pass2<2>, m));
  PF_CUDA(c, allow_smem(k_split_rows<true>, m));
  PF_CUDA(c, allow_smem(k_split_cols<true>, m));
  if (c->fast) PF_CUDA(c, c->fl.set_attrs(m, m));
  return PF_OK;
}

bool fast_table(int n, FastLaunch* fl) {
  switch (n) {
    case 32: *fl = pf_fast_table_32(); return true;
    case 48: *fl = pf_fast_table_48(); return true;
    case 64: *fl = pf_fast_table_64(); return true;
    case 96: *fl = pf_fast_table_96(); return true;
    case 128: *fl = pf_fast_table_128(); return true;
    case 160: *fl = pf_fast_table_160(); return true;
    case 192: *fl = pf_fast_table_192(); return true;
    default: return false;
  }
}

// (z, y, points in the sphere) of every row with cz^2 + cy^2 <= re^2, z-major
int build_rows(pf_ctx* c, int re, int4** dptr, int* count) {
  std::vector<int4> rows;
  const long long re2 = (long long)re * re;
  for (int z = 0; z < c->nz; ++z) {
    const int cz = (2 * z <= c->nz) ? z : z - c->nz;
    for (int y = 0; y < c->ny; ++y) {
      const int cy = (2 * y <= c->ny) ? y : y - c->ny;
      const long long rem = re2 - (long long)cz * cz - (long long)cy * cy;
      if (rem < 0) continue;
      long long xr = (long long)std::sqrt((double)rem);
      while (xr * xr > rem) --xr;
      while ((xr + 1) * (xr + 1) <= rem) ++xr;
      const int cnt = (2 * xr + 1 >= c->nx) ? c->nx : (int)(2 * xr + 1);
      rows.push_back(make_int4(z, y, cnt, 0));
    }
  }
  if (*dptr) cudaFree(*dptr);
  *dptr = nullptr;
  *count = (int)rows.size();
  if (rows.empty()) return PF_OK;
  int rc = alloc(c, (void**)dptr, rows.size() * sizeof(int4));
  if (rc) return rc;
  PF_CUDA(c, cudaMemcpy(*dptr, rows.data(), rows.size() * sizeof(int4), cudaMemcpyHostToDevice));
  return PF_OK;
}

int upload_double_as_float(pf_ctx* c, float* dst, const double* src, long long n) {
  std::vector<float> tmp((size_t)n);
  for (long long i = 0; i < n; ++i) tmp[i] = (float)src[i];
  PF_CUDA(c, cudaMemcpyAsync(dst, tmp.data(), n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  PF_CUDA(c, cudaStreamSynchronize(c->stream));
  return PF_OK;
}

constexpr int kSplitRows = 16;   // rows per tile of the split pass 2 (steps 2a, 2c)
constexpr int kSplitCols = 16;   // columns per tile (step 2b)

// pass 2 in three steps through global memory (planes larger than shared memory);
// tc: DFT stages on the tensor cores (split-bf16x3)
// The tensor-core stages hold at most 8 * kMmaGroups butterflies per warp in a
// chunk: with 256-thread blocks a line of nb = L/R <= 128 butterflies always fits.
constexpr int kTensorDftMaxEdge = 256;

int launch_split_pass2(pf_ctx* c, const Geometry& g, int npairs, int nfield, int mode, float2* out, float scale,
                       bool tc = false) {
  const size_t srow = ((size_t)c->ny + (size_t)kSplitRows * (c->ny + kPad)) * sizeof(float2);
  const size_t scol = ((size_t)c->nz + (size_t)c->nz * (kSplitCols + kPad)) * sizeof(float2);
  SplitRowsParams pr{g, c->py, c->twy, c->buf, nfield, kSplitRows, 0, buf_extent(c)};
  dim3 gr((g.nvz + kSplitRows - 1) / kSplitRows, c->nx, npairs * nfield);
  if (tc) k_split_rows<true><<<gr, kThreadsLine, srow, c->stream>>>(pr);
  else k_split_rows<false><<<gr, kThreadsLine, srow, c->stream>>>(pr);
  PF_CUDA(c, cudaGetLastError());
  SplitColsParams pc{g, c->pz, c->twz, c->buf, c->spec, c->spec + c->N, nfield, kSplitCols, mode, out, scale,
                     buf_extent(c), c->N, out ? 2 * c->N : 0};
  dim3 gc((c->ny + kSplitCols - 1) / kSplitCols, c->nx, npairs * nfield);
  if (tc) k_split_cols<true><<<gc, kThreadsLine, scol, c->stream>>>(pc);
  else k_split_cols<false><<<gc, kThreadsLine, scol, c->stream>>>(pc);
  PF_CUDA(c, cudaGetLastError());
  if (mode == 0) {
    SplitRowsParams pi{g, c->py, c->twy, c->buf, nfield, kSplitRows, 1, buf_extent(c)};
    dim3 gi((c->nz + kSplitRows - 1) / kSplitRows, c->nx, npairs * nfield);
    if (tc) k_split_rows<true><<<gi, kThreadsLine, srow, c->stream>>>(pi);
    else k_split_rows<false><<<gi, kThreadsLine, srow, c->stream>>>(pi);
    PF_CUDA(c, cudaGetLastError());
  }
  return PF_OK;
}

// forward transforms of two real device fields -> spectra [2][kx][kz][ky] * scale
int forward_two_fields(pf_ctx* c, const float* in0, const float* in1, int square1, float2* out, float scale) {
  int rc = ensure_buf(c, 1);
  if (rc) return rc;
  Geometry gfull = c->g;
  gfull.nvz = c->nz;
  gfull.zlo = c->nz - 1;
  const int ty = c->ty1;
  FwdXParams fx{gfull, c->px, c->twx, in0, in1, square1, c->buf, ty, buf_extent(c)};
  dim3 g1(c->nz, (c->ny + ty - 1) / ty, 1);
  k_fwd_x_real<<<g1, kThreadsLine, line_smem(c->nx, 3, ty), c->stream>>>(fx);
  PF_CUDA(c, cudaGetLastError());
  Pass2Params p2{};
  p2.g = gfull;
  p2.py = c->py;
  p2.pz = c->pz;
  p2.twy = c->twy;
  p2.twz = c->twz;
  p2.buf = c->buf;
  p2.nfield = 2;
  p2.mode = 1;
  p2.out = out;
  p2.scale = scale;
  p2.buf_len = buf_extent(c);
  p2.out_len = 2 * c->N;
  dim3 g2(c->nx, 2, 1);
  if (c->split) {
    int rc2 = launch_split_pass2(c, gfull, 1, 2, 1, out, scale);
    if (rc2) return rc2;
  } else if (c->fast) {
    c->fl.pass2(p2, 0, g2, plane_smem(c->ny, c->nz), c->stream);
  } else {
    k_pass2<false><<<g2, kThreadsPlane, plane_smem(c->ny, c->nz), c->stream>>>(p2);
  }
  PF_CUDA(c, cudaGetLastError());
  PF_CUDA(c, cudaStreamSynchronize(c->stream));
  return PF_OK;
}

}  // namespace

#ifdef PF_BOUNDS_CHECK
int pf_check_register(int (*take)(unsigned long long* first, unsigned long long* count)) {
  std::lock_guard<std::mutex> lock(check_mutex());
  check_units().push_back(take);
  return (int)check_units().size();
}
#endif

extern "C" {

int pf_global_error(char* buf, size_t len) {
  if (!buf || !len) return PF_E_ARG;
  snprintf(buf, len, "%s", g_err);
  return PF_OK;
}

int pf_last_error(const pf_ctx* ctx, char* buf, size_t len) {
  if (!buf || !len) return PF_E_ARG;
  snprintf(buf, len, "%s", ctx ? ctx->err : g_err);
  return PF_OK;
}

pf_ctx* pf_create(int nz, int ny, int nx, int device, int* status) {
  auto ret = [&](int code) -> pf_ctx* {
    if (status) *status = code;
    return nullptr;
  };
  if (nz < 1 || ny < 1 || nx < 1) {
    set_global_error("grid shape must be positive, got (%d, %d, %d)", nz, ny, nx);
    return ret(PF_E_ARG);
  }
  if (nz > 2048 || ny > 2048 || nx > 2048) {
    set_global_error("grid edges are limited to 2048, got (%d, %d, %d)", nz, ny, nx);
    return ret(PF_E_SHAPE);
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    set_global_error("CUDA device %d not available (%d devices)", device, ndev);
    return ret(PF_E_CUDA);
  }
  DeviceGuard guard(device);
  pf_ctx* c = new pf_ctx();
  c->device = device;
  c->nz = nz;
  c->ny = ny;
  c->nx = nx;
  c->N = (long long)nz * ny * nx;
  if (!make_plan(nx, &c->px) || !make_plan(ny, &c->py) || !make_plan(nz, &c->pz)) {
    set_global_error("grid (%d, %d, %d): every edge must factor into 2, 3, 5 and 7", nz, ny, nx);
    delete c;
    return ret(PF_E_SHAPE);
  }
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  c->max_smem = prop.sharedMemPerBlockOptin;
  c->num_sms = prop.multiProcessorCount;
  c->split = plane_smem(ny, nz) > c->max_smem;
  c->rmax = std::min(nz, std::min(ny, nx)) / 2;
  if (nz == ny && ny == nx) {
    FastLaunch fl{};
    if (fast_table(nx, &fl) && (!c->split || fl.cluster_plane)) {
      c->fast = true;
      c->fl = fl;
    }
  }
  choose_tiles(c);
  int rc = PF_OK;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(c, PF_E_CUDA, "stream creation failed");
  c->stream = c->own_stream;
  const size_t N = (size_t)c->N;
  if (!rc) rc = alloc(c, (void**)&c->twx, nx * sizeof(float2));
  if (!rc) rc = alloc(c, (void**)&c->twy, ny * sizeof(float2));
  if (!rc) rc = alloc(c, (void**)&c->twz, nz * sizeof(float2));
  if (!rc) rc = alloc(c, (void**)&c->tmpl, N * sizeof(float));
  if (!rc) rc = alloc(c, (void**)&c->mask, N * sizeof(float));
  if (!rc) rc = alloc(c, (void**)&c->lcc_mask, N);
  if (!rc) rc = alloc(c, (void**)&c->spec, 2 * N * sizeof(float2));
  if (!rc) rc = alloc(c, (void**)&c->lcc, N * sizeof(float));
  if (!rc) rc = alloc(c, (void**)&c->rot, N * sizeof(int));
  if (!rc) rc = ensure_buf(c, c->pairs);
  if (!rc) rc = alloc(c, (void**)&c->d_err, sizeof(int));
  if (!rc && cudaMemset(c->d_err, 0, sizeof(int)) != cudaSuccess) rc = fail(c, PF_E_CUDA, "memset failed");
  if (!rc) {
    auto tx = twiddles(nx), ty = twiddles(ny), tz = twiddles(nz);
    if (cudaMemcpy(c->twx, tx.data(), nx * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(c->twy, ty.data(), ny * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(c->twz, tz.data(), nz * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess)
      rc = fail(c, PF_E_CUDA, "twiddle upload failed");
  }
  if (!rc) rc = set_smem_limits(c);
  if (!rc && (cudaMemset(c->lcc, 0, N * sizeof(float)) != cudaSuccess ||
              cudaMemset(c->rot, 0, N * sizeof(int)) != cudaSuccess))
    rc = fail(c, PF_E_CUDA, "memset failed");
  compute_geometry(c, c->rmax);
  if (rc) {
    snprintf(g_err, sizeof(g_err), "%s", c->err);
    pf_destroy(c);
    return ret(rc);
  }
  if (status) *status = PF_OK;
  return c;
}

int pf_destroy(pf_ctx* c) {
  if (!c) return PF_E_ARG;
  DeviceGuard guard(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  collect_events(c);
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  c->own_stream = nullptr;
  void* ptrs[] = {c->twx, c->twy, c->twz, c->tmpl, c->mask, c->lcc_mask, c->spec, c->lcc, c->rot, c->buf, c->rots, c->rotd,
                  c->rows_reach, c->rows_full, c->tmpl_pairs, c->part_lcc, c->part_rot, c->rotmax, c->d_err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete c;
  return PF_OK;
}

int pf_set_stream(pf_ctx* c, void* stream) {
  if (!c) return PF_E_ARG;
  DeviceGuard guard(c->device);
  PF_CUDA(c, cudaStreamSynchronize(c->stream));
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return PF_OK;
}

int pf_set_target(pf_ctx* c, const double* target, const uint8_t* lcc_mask) {
  if (!c || !target || !lcc_mask) return fail(c, PF_E_ARG, "pf_set_target: null argument");
  DeviceGuard guard(c->device);
  const long long N = c->N;
  float* dt = nullptr;
  int rc = alloc(c, (void**)&dt, N * sizeof(float));
  if (rc) return rc;
  rc = upload_double_as_float(c, dt, target, N);
  if (!rc && cudaMemcpy(c->lcc_mask, lcc_mask, N, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = fail(c, PF_E_CUDA, "lcc mask upload failed");
  if (!rc) rc = forward_two_fields(c, dt, nullptr, 1, c->spec, (float)(1.0 / (double)N));
  cudaFree(dt);
  if (!rc) c->have_target = true;
  return rc;
}

int pf_set_template_mask(pf_ctx* c, const double* tmpl, const double* mask, double norm_factor, int rmax) {
  if (!c || !tmpl || !mask) return fail(c, PF_E_ARG, "pf_set_template_mask: null argument");
  if (!(norm_factor > 0)) return fail(c, PF_E_ARG, "norm_factor must be positive (zero-filled mask)");
  if (rmax < 0 || 2 * rmax > std::min(c->nz, std::min(c->ny, c->nx)))
    return fail(c, PF_E_ARG, "rmax %d outside [0, min(shape)//2]", rmax);
  DeviceGuard guard(c->device);
  int rc = upload_double_as_float(c, c->tmpl, tmpl, c->N);
  if (!rc) rc = upload_double_as_float(c, c->mask, mask, c->N);
  if (rc) return rc;
  c->rmax = rmax;
  c->norm_factor = (float)norm_factor;
  // radius of the data support (minimal-image distance of any nonzero voxel)
  double rs2 = -1.0;
  for (int z = 0; z < c->nz; ++z) {
    const int cz = (2 * z <= c->nz) ? z : z - c->nz;
    for (int y = 0; y < c->ny; ++y) {
      const int cy = (2 * y <= c->ny) ? y : y - c->ny;
      const long long row = ((long long)z * c->ny + y) * c->nx;
      for (int x = 0; x < c->nx; ++x) {
        if (tmpl[row + x] != 0.0 || mask[row + x] != 0.0) {
          const int cx = (2 * x <= c->nx) ? x : x - c->nx;
          const double d2 = (double)cz * cz + (double)cy * cy + (double)cx * cx;
          if (d2 > rs2) rs2 = d2;
        }
      }
    }
  }
  const int nmin = std::min(c->nz, std::min(c->ny, c->nx));
  const double rs = rs2 < 0 ? 0.0 : std::sqrt(rs2);
  // a rotated sample at |p| > rs + sqrt(3) only touches voxels farther than rs
  // (as long as the support stays clear of the periodic boundary)
  int reff = rmax;
  if (rs + 1.0 < nmin / 2.0) reff = std::min(rmax, (int)std::floor(rs + 1.7320508075688772 + 1e-6) + 1);
  c->reff_data = reff;
  compute_geometry(c, reff);
  if (c->fast) {
    int rc2 = build_rows(c, std::min(rmax, reff), &c->rows_reach, &c->nrows_reach);
    if (!rc2) rc2 = build_rows(c, rmax, &c->rows_full, &c->nrows_full);
    if (!rc2 && !c->tmpl_pairs) rc2 = alloc(c, (void**)&c->tmpl_pairs, c->N * sizeof(float2));
    if (rc2) return rc2;
    k_make_pairs<<<(unsigned)std::min<long long>((c->N + 255) / 256, 8192), 256, 0, c->stream>>>(c->tmpl, c->tmpl_pairs,
                                                                                             c->nx, c->N);
    PF_CUDA(c, cudaGetLastError());
    PF_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  c->have_template = true;
  return PF_OK;
}

int pf_set_rotations(pf_ctx* c, const double* rotmats, int64_t nrot) {
  if (!c || (!rotmats && nrot > 0) || nrot < 0) return fail(c, PF_E_ARG, "pf_set_rotations: bad arguments");
  if (nrot > (int64_t)0x7fffffff) return fail(c, PF_E_ARG, "too many rotations");
  DeviceGuard guard(c->device);
  if (nrot > c->rot_cap) {
    if (c->rots) cudaFree(c->rots);
    if (c->rotd) cudaFree(c->rotd);
    c->rots = nullptr;
    c->rotd = nullptr;
    c->rot_cap = 0;
    int rc = alloc(c, (void**)&c->rots, std::max<int64_t>(nrot, 1) * sizeof(RotFixed));
    if (!rc) rc = alloc(c, (void**)&c->rotd, std::max<int64_t>(nrot, 1) * 9 * sizeof(double));
    if (rc) return rc;
    c->rot_cap = nrot;
  }
  std::vector<RotFixed> fx((size_t)nrot);
  for (int64_t i = 0; i < nrot; ++i) {
    for (int k = 0; k < 9; ++k)
      if (!std::isfinite(rotmats[9 * i + k]) || std::fabs(rotmats[9 * i + k]) > 2.0)
        return fail(c, PF_E_ARG, "rotation %lld element %d is not a rotation-matrix entry", (long long)i, k);
    fx[i] = to_fixed(rotmats + 9 * i);
  }
  if (nrot > 0) {
    PF_CUDA(c, cudaMemcpyAsync(c->rots, fx.data(), nrot * sizeof(RotFixed), cudaMemcpyHostToDevice, c->stream));
    PF_CUDA(c, cudaMemcpyAsync(c->rotd, rotmats, nrot * 9 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    PF_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  c->nrot = nrot;
  return PF_OK;
}

int pf_set_results(pf_ctx* c, const float* lcc, const int32_t* rot) {
  if (!c || !lcc || !rot) return fail(c, PF_E_ARG, "pf_set_results: null argument");
  DeviceGuard guard(c->device);
  PF_CUDA(c, cudaMemcpyAsync(c->lcc, lcc, c->N * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  PF_CUDA(c, cudaMemcpyAsync(c->rot, rot, c->N * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  PF_CUDA(c, cudaStreamSynchronize(c->stream));
  return PF_OK;
}

int pf_debug_fail_alloc(int64_t after) {
  g_fail_alloc_after.store(after < 0 ? -1 : (long long)after);
  return PF_OK;
}

int pf_debug_bounds(int device, uint64_t* first, uint64_t* count) {
#ifdef PF_BOUNDS_CHECK
  if (!first || !count) return fail(nullptr, PF_E_ARG, "pf_debug_bounds: null output pointer");
  DeviceGuard guard(device);
  PF_CUDA(nullptr, cudaDeviceSynchronize());
  *first = 0;
  *count = 0;
  std::lock_guard<std::mutex> lock(check_mutex());
  for (CheckTake take : check_units()) {
    unsigned long long f = 0, n = 0;
    if (take(&f, &n)) return fail(nullptr, PF_E_CUDA, "pf_debug_bounds: cannot read a check word");
    if (!*first) *first = f;
    *count += n;
  }
  return PF_OK;
#else
  (void)device;
  (void)first;
  (void)count;
  return fail(nullptr, PF_E_UNSUPPORTED, "pf_debug_bounds: library built without bounds checks");
#endif
}

int pf_debug_buffer_extent(pf_ctx* c, int64_t elements) {
  if (!c) return PF_E_ARG;
#ifdef PF_BOUNDS_CHECK
  c->debug_buf_extent = elements < 0 ? -1 : (long long)elements;
  return PF_OK;
#else
  (void)elements;
  return fail(c, PF_E_UNSUPPORTED, "pf_debug_buffer_extent: library built without bounds checks");
#endif
}

int pf_bounds_checked(void) {
#ifdef PF_BOUNDS_CHECK
  return 1;
#else
  return 0;
#endif
}

int pf_reset_results(pf_ctx* c) {
  if (!c) return PF_E_ARG;
  DeviceGuard guard(c->device);
  PF_CUDA(c, cudaMemsetAsync(c->lcc, 0, c->N * sizeof(float), c->stream));
  PF_CUDA(c, cudaMemsetAsync(c->rot, 0, c->N * sizeof(int), c->stream));
  return PF_OK;
}

int pf_scan_resident(pf_ctx* c, int64_t first, int64_t count, int64_t rot_offset, int flags) {
  if (!c) return fail(c, PF_E_ARG, "null context");
  if (!c->have_target || !c->have_template) return fail(c, PF_E_STATE, "set the target and the template/mask first");
  if (first < 0 || count < 0 || first + count > c->nrot) return fail(c, PF_E_ARG, "rotation range outside the uploaded set");
  if (rot_offset + first + count > (int64_t)0x7fffffff) return fail(c, PF_E_ARG, "rotation index overflows int32");
  if ((flags & PF_FLAG_TENSOR_DFT) && std::max(c->nx, std::max(c->ny, c->nz)) > kTensorDftMaxEdge)
    return fail(c, PF_E_ARG, "PF_FLAG_TENSOR_DFT: grid edges are limited to %d", kTensorDftMaxEdge);
  DeviceGuard guard(c->device);
  int rc = ensure_buf(c, c->pairs);
  if (rc) return rc;
  if (!(flags & PF_FLAG_ACCUMULATE)) {
    rc = pf_reset_results(c);
    if (rc) return rc;
  }
  if (flags & PF_FLAG_ROT_MAX) {
    if (c->rotmax_cap < c->nrot) {
      if (c->rotmax) cudaFree(c->rotmax);
      c->rotmax = nullptr;
      c->rotmax_cap = 0;
      rc = alloc(c, (void**)&c->rotmax, std::max<long long>(c->nrot, 1) * sizeof(unsigned long long));
      if (rc) return rc;
      c->rotmax_cap = c->nrot;
      PF_CUDA(c, cudaMemsetAsync(c->rotmax, 0, c->rotmax_cap * sizeof(unsigned long long), c->stream));
    }
    if (!(flags & PF_FLAG_ACCUMULATE) && count > 0)
      PF_CUDA(c, cudaMemsetAsync(c->rotmax + first, 0, count * sizeof(unsigned long long), c->stream));
  }
  Geometry g = c->g;
  if (flags & PF_FLAG_NO_PRUNE) {
    Geometry full = g;
    full.reff = c->rmax;
    const int re = c->rmax;
    if (2 * re + 1 >= c->nz) { full.nvz = c->nz; full.zlo = c->nz - 1; }
    else { full.nvz = 2 * re + 1; full.zlo = re; }
    g = full;
  }
  const int P = c->pairs;
  const int ty1 = c->ty1, ty3 = c->ty3;
  const size_t s1 = line_smem(c->nx, 3, ty1), s3 = line_smem(c->nx, 3, ty3), s2 = plane_smem(c->ny, c->nz);
  const bool tc = (flags & PF_FLAG_TENSOR_DFT) != 0;
  const bool tc05 = tc && (flags & PF_FLAG_TENSOR_TC05) != 0;
  const bool fast = c->fast && !(flags & PF_FLAG_GENERIC) && !tc;
  if (tc05) {
    if (c->split || pass2_tc05_smem(s2) > c->max_smem)
      return fail(c, PF_E_ARG, "PF_FLAG_TENSOR_TC05: the (z, y) plane and the tcgen05 operands exceed shared memory");
    const int zero = 0;
    PF_CUDA(c, cudaMemcpyToSymbolAsync(g_tc05_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, c->stream));
  }
  const int re = std::min(g.rmax, g.reff);
  const int re2 = re * re;
  const int64_t end = first + count;
  for (int64_t r0 = first; r0 < end; r0 += 2LL * P) {
    const int npairs = (int)std::min<int64_t>(P, (end - r0 + 1) / 2);
    const bool full = (flags & PF_FLAG_NO_PRUNE) != 0;
    Pass1Params p1{g, c->px, GatherSrc{c->tmpl, c->mask, c->tmpl_pairs}, c->twx, c->rots, c->rotd, r0, end, c->buf, ty1,
                   full ? c->rows_full : c->rows_reach, full ? c->nrows_full : c->nrows_reach, buf_extent(c)};
    rc = timed_launch(c, 0, [&] {
      if (fast) {
        if (p1.nrows == 0) return 0;
        dim3 g1((p1.nrows + ty1 - 1) / ty1, 1, npairs);
        c->fl.pass1(p1, re2, g1, s1, c->stream);
        return 1;
      } else {
        dim3 g1(g.nvz, (c->ny + ty1 - 1) / ty1, npairs);
        if (tc) k_pass1<true><<<g1, kThreadsLine, s1, c->stream>>>(p1);
        else k_pass1<false><<<g1, kThreadsLine, s1, c->stream>>>(p1);
        return 1;
      }
    });
    if (rc) return rc;
    Pass2Params p2{};
    p2.g = g;
    p2.py = c->py;
    p2.pz = c->pz;
    p2.twy = c->twy;
    p2.twz = c->twz;
    p2.buf = c->buf;
    p2.s1 = c->spec;
    p2.s2 = c->spec + c->N;
    p2.nfield = 3;
    p2.mode = 0;
    p2.buf_len = buf_extent(c);
    p2.spec_len = c->N;
    dim3 g2(c->nx, 3, npairs);
    rc = timed_launch(c, 1, [&] {
      if (fast) {
        c->fl.pass2(p2, re2, g2, s2, c->stream);
        return 1;
      }
      if (c->split) {
        launch_split_pass2(c, g, npairs, 3, 0, nullptr, 1.0f, tc);   // rows, columns, rows
        return 3;
      }
      if (tc05) k_pass2<2><<<g2, kThreadsPlane, pass2_tc05_smem(s2), c->stream>>>(p2);
      else if (tc) k_pass2<true><<<g2, kThreadsPlane, s2, c->stream>>>(p2);
      else k_pass2<false><<<g2, kThreadsPlane, s2, c->stream>>>(p2);
      return 1;
    });
    if (rc) return rc;
    Pass3Params p3{g, c->px, c->twx, c->buf, npairs, r0, end, rot_offset, c->lcc_mask, c->norm_factor,
                   c->lcc, c->rot, ty3, (flags & PF_FLAG_FP64_NORM) ? 1 : 0};
    if (flags & PF_FLAG_ROT_MAX) {
      p3.rotmax = c->rotmax;
      p3.rotmax_len = c->rotmax_cap;
    }
    p3.buf_len = buf_extent(c);
    dim3 g3(c->nz, (c->ny + ty3 - 1) / ty3, 1);
    // Each pass-3 block runs through all pairs of the batch, so a grid of a
    // few waves (or of fewer tiles than the GPU holds blocks) leaves much of
    // its last wave idle; splitting the pairs over up to kPass3MaxParts blocks
    // per tile (merged afterwards) evens the waves out.  A split is taken only
    // where it fills the waves by more than 5 points over the fewer parts.
    if (fast && npairs >= 4 && c->num_sms > 0) {
      const double slots = (double)kPass3BlocksPerSm * c->num_sms;
      auto eff = [&](double blocks) { const double w = blocks / slots; return w / std::ceil(w); };
      const double tiles = (double)g3.x * g3.y;
      int parts = 1;
      for (int k = 2; k <= kPass3MaxParts && 2 * k <= npairs; ++k)
        if (eff(k * tiles) > eff(parts * tiles) + 0.05) parts = k;
      if (parts > 1) {
        rc = ensure_part(c, parts - 1);
        if (rc) return rc;
        g3.z = parts;
        p3.part_lcc = c->part_lcc;
        p3.part_rot = c->part_rot;
      }
    }
    const size_t s3f = pass3_smem(c->nx, ty3, npairs > 1 ? 2 : 1);
    rc = timed_launch(c, 2, [&] {
      if (fast) {
        const bool tm = PF_P3_TMA && ensure_tile_map(c, ty3);
        p3.tma = tm ? 1 : 0;
        p3.err = c->d_err;
        c->fl.pass3(p3, tm ? &c->tmap3 : nullptr, g3, s3f, c->stream);
        if (g3.z == 1) return 1;
        k_combine_parts<<<(unsigned)std::min<long long>((c->N + 255) / 256, 4 * 1024), 256, 0, c->stream>>>(
            c->part_lcc, c->part_rot, (int)g3.z - 1, c->lcc, c->rot, c->N);
        return 2;
      }
      if (tc) k_pass3<true><<<g3, kThreadsLine, s3, c->stream>>>(p3);
      else k_pass3<false><<<g3, kThreadsLine, s3, c->stream>>>(p3);
      return 1;
    });
    if (rc) return rc;
  }
  if (tc05) {   // a tensor-core wait that ran out in any block of the plane pass
    int err = 0;
    PF_CUDA(c, cudaMemcpyFromSymbolAsync(&err, g_tc05_error, sizeof(int), 0, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(c, cudaStreamSynchronize(c->stream));
    if (err) return fail(c, PF_E_CUDA, "PF_FLAG_TENSOR_TC05: a wait for the tensor-core products ran out");
  }
  return PF_OK;
}

int pf_get_results(pf_ctx* c, float* out_lcc, int32_t* out_rot) {
  if (!c || !out_lcc || !out_rot) return fail(c, PF_E_ARG, "pf_get_results: null argument");
  DeviceGuard guard(c->device);
  PF_CUDA(c, cudaMemcpyAsync(out_lcc, c->lcc, c->N * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  PF_CUDA(c, cudaMemcpyAsync(out_rot, c->rot, c->N * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  PF_CUDA(c, cudaStreamSynchronize(c->stream));
  if (c->profiling) collect_events(c);
  return check_tile_error(c);
}

int pf_get_rotation_best(pf_ctx* c, float* value, int32_t* voxel, int64_t first, int64_t count) {
  if (!c || (count > 0 && !value && !voxel) || first < 0 || count < 0)
    return fail(c, PF_E_ARG, "pf_get_rotation_best: bad arguments");
  if (first + count > c->rotmax_cap) return fail(c, PF_E_STATE, "no per-rotation maxima for that range (scan with PF_FLAG_ROT_MAX)");
  if (count == 0) return PF_OK;
  DeviceGuard guard(c->device);
  std::vector<unsigned long long> keys((size_t)count);
  PF_CUDA(c, cudaMemcpyAsync(keys.data(), c->rotmax + first, count * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, c->stream));
  PF_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int64_t i = 0; i < count; ++i) {
    const unsigned long long key = keys[(size_t)i];
    const unsigned int k = (unsigned int)(key >> 32);
    float f = -INFINITY;
    if (k) {
      const unsigned int u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
      std::memcpy(&f, &u, sizeof f);
    }
    if (value) value[i] = f;
    if (voxel) voxel[i] = k ? (int32_t)(unsigned int)(key & 0xffffffffu) : -1;
  }
  return PF_OK;
}

int pf_get_rotation_max(pf_ctx* c, float* out, int64_t first, int64_t count) {
  if (!c || (!out && count > 0)) return fail(c, PF_E_ARG, "pf_get_rotation_max: bad arguments");
  return pf_get_rotation_best(c, out, nullptr, first, count);
}

int pf_synchronize(pf_ctx* c) {
  if (!c) return PF_E_ARG;
  DeviceGuard guard(c->device);
  PF_CUDA(c, cudaStreamSynchronize(c->stream));
  if (c->profiling) collect_events(c);
  return check_tile_error(c);
}

int pf_scan(pf_ctx* c, const double* rotmats, int64_t nrot, int64_t rot_offset, float* out_lcc, int32_t* out_rot,
            int flags) {
  if (!c) return fail(c, PF_E_ARG, "null context");
  int rc = pf_set_rotations(c, rotmats, nrot);
  if (!rc) rc = pf_scan_resident(c, 0, nrot, rot_offset, flags & ~PF_FLAG_ACCUMULATE);
  if (!rc) rc = pf_get_results(c, out_lcc, out_rot);
  return rc;
}

int pf_set_tuning(pf_ctx* c, int pairs, int rows1, int rows3) {
  if (!c) return PF_E_ARG;
  if (pairs < 0 || rows1 < 0 || rows3 < 0) return fail(c, PF_E_ARG, "tuning values must be >= 0");
  auto ok_rows = [&](int ty) {
    return (long long)ty * c->nx <= (long long)kMaxVoxPerThread * kThreadsLine &&
           line_smem(c->nx, 3, ty) <= std::max(line_smem(c->nx, 3, 16), (size_t)48 * 1024);
  };
  if (rows1 && (!ok_rows(rows1) || rows1 > 32)) return fail(c, PF_E_ARG, "rows_pass1 %d too large for nx %d", rows1, c->nx);
  if (rows3 && (!ok_rows(rows3) || (long long)rows3 * c->nx > max_vox3(c)))
    return fail(c, PF_E_ARG, "rows_pass3 %d too large for nx %d", rows3, c->nx);
  if (rows3 && ((rows3 & (rows3 - 1)) || (c->fast && rows3 < 2)))
    return fail(c, PF_E_ARG, "rows_pass3 must be a power of two (>= 2 for this grid)");
  if (pairs) {
    DeviceGuard guard(c->device);
    cudaStreamSynchronize(c->stream);
    int rc = ensure_buf(c, pairs);
    if (rc) return rc;
    c->pairs = pairs;
  }
  if (rows1) c->ty1 = rows1;
  if (rows3) c->ty3 = rows3;
  return PF_OK;
}

int pf_autotune(pf_ctx* c, int64_t trial_rotations, int* best_pairs, int* best_rows1, int* best_rows3,
                double* best_ms) {
  if (!c) return PF_E_ARG;
  if (!c->have_target || !c->have_template || c->nrot < 1)
    return fail(c, PF_E_STATE, "autotune needs the target, the template/mask and a rotation set");
  DeviceGuard guard(c->device);
  const int64_t trial = std::max<int64_t>(1, std::min<int64_t>(trial_rotations > 0 ? trial_rotations : 512, c->nrot));
  cudaEvent_t e0, e1;
  PF_CUDA(c, cudaEventCreate(&e0));
  PF_CUDA(c, cudaEventCreate(&e1));
  const bool prof = c->profiling;
  c->profiling = false;
  auto time_cfg = [&](int pairs, int r1, int r3, float* ms) -> int {
    int rc = pf_set_tuning(c, pairs, r1, r3);
    if (rc) return rc;
    rc = pf_scan_resident(c, 0, trial, 0, 0);   // warm-up (also allocates)
    if (rc) return rc;
    float best = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0, c->stream);
      rc = pf_scan_resident(c, 0, trial, 0, 0);
      if (rc) return rc;
      cudaEventRecord(e1, c->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) return fail(c, PF_E_CUDA, "autotune timing failed");
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      best = std::min(best, t);
    }
    *ms = best;
    return PF_OK;
  };
  int bp = c->pairs, b1 = c->ty1, b3 = c->ty3;
  float bms = 1e30f;
  int rc = time_cfg(bp, b1, b3, &bms);
  // pairs per batch, capped by free device memory (half of what is free)
  size_t freeb = 0, totalb = 0;
  cudaMemGetInfo(&freeb, &totalb);
  const size_t per_pair = 3ull * c->N * sizeof(float2);
  const int pair_cands[] = {1, 2, 4, 8, 16, 24, 32, 48, 64, 96, 128};
  for (int pc : pair_cands) {
    if (rc) break;
    if (pc == bp || (size_t)pc * per_pair > (size_t)c->buf_pairs * per_pair + freeb / 2) continue;
    if (2LL * pc > 4 * trial) continue;
    float ms;
    rc = time_cfg(pc, b1, b3, &ms);
    if (!rc && ms < bms) { bms = ms; bp = pc; }
  }
  const int row_cands[] = {2, 4, 8, 16, 32};
  for (int r1 : row_cands) {
    if (rc) break;
    if (r1 == b1 || (long long)r1 * c->nx > (long long)kMaxVoxPerThread * kThreadsLine ||
        line_smem(c->nx, 3, r1) > std::max(line_smem(c->nx, 3, 16), (size_t)48 * 1024))
      continue;
    float ms;
    rc = time_cfg(bp, r1, b3, &ms);
    if (!rc && ms < bms) { bms = ms; b1 = r1; }
  }
  for (int r3 : row_cands) {
    if (rc) break;
    if (r3 == b3 || (long long)r3 * c->nx > max_vox3(c) ||
        line_smem(c->nx, 3, r3) > std::max(line_smem(c->nx, 3, 16), (size_t)48 * 1024))
      continue;
    float ms;
    rc = time_cfg(bp, b1, r3, &ms);
    if (!rc && ms < bms) { bms = ms; b3 = r3; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->profiling = prof;
  if (rc) return rc;
  rc = pf_set_tuning(c, bp, b1, b3);
  if (rc) return rc;
  rc = pf_reset_results(c);
  if (best_pairs) *best_pairs = bp;
  if (best_rows1) *best_rows1 = b1;
  if (best_rows3) *best_rows3 = b3;
  if (best_ms) *best_ms = bms;
  return rc;
}

int pf_get_tuning(const pf_ctx* c, int* pairs, int* rows1, int* rows3) {
  if (!c) return PF_E_ARG;
  if (pairs) *pairs = c->pairs;
  if (rows1) *rows1 = c->ty1;
  if (rows3) *rows3 = c->ty3;
  return PF_OK;
}

int pf_get_geometry(const pf_ctx* c, int* reff, int* valid_planes, int* rmax) {
  if (!c) return PF_E_ARG;
  if (reff) *reff = c->g.reff;
  if (valid_planes) *valid_planes = c->g.nvz;
  if (rmax) *rmax = c->rmax;
  return PF_OK;
}

int pf_set_profiling(pf_ctx* c, int enable) {
  if (!c) return PF_E_ARG;
  DeviceGuard guard(c->device);
  cudaStreamSynchronize(c->stream);
  collect_events(c);
  c->profiling = enable != 0;
  for (int i = 0; i < 3; ++i) {
    c->ms[i] = 0;
    c->launches[i] = 0;
  }
  return PF_OK;
}

int pf_get_kernel_times(pf_ctx* c, double* ms, int64_t* launches) {
  if (!c || !ms || !launches) return PF_E_ARG;
  DeviceGuard guard(c->device);
  cudaStreamSynchronize(c->stream);
  collect_events(c);
  for (int i = 0; i < 3; ++i) {
    ms[i] = c->ms[i];
    launches[i] = c->launches[i];
  }
  return PF_OK;
}

int pf_fft3d(pf_ctx* c, const float* in, float* out) {
  if (!c || !in || !out) return fail(c, PF_E_ARG, "pf_fft3d: null argument");
  DeviceGuard guard(c->device);
  const long long N = c->N;
  float* din = nullptr;
  float2* dout = nullptr;
  int rc = alloc(c, (void**)&din, N * sizeof(float));
  if (!rc) rc = alloc(c, (void**)&dout, 2 * N * sizeof(float2));
  if (!rc && cudaMemcpy(din, in, N * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    rc = fail(c, PF_E_CUDA, "upload failed");
  if (!rc) rc = forward_two_fields(c, din, nullptr, 0, dout, 1.0f);
  std::vector<float2> h;
  if (!rc) {
    h.resize((size_t)N);
    if (cudaMemcpy(h.data(), dout, N * sizeof(float2), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(c, PF_E_CUDA, "download failed");
  }
  if (!rc) {
    // device layout [kx][kz][ky] -> natural [kz][ky][kx]
    for (int kx = 0; kx < c->nx; ++kx)
      for (int kz = 0; kz < c->nz; ++kz)
        for (int ky = 0; ky < c->ny; ++ky) {
          const float2 v = h[((size_t)kx * c->nz + kz) * c->ny + ky];
          const size_t o = ((size_t)kz * c->ny + ky) * c->nx + kx;
          out[2 * o] = v.x;
          out[2 * o + 1] = v.y;
        }
  }
  if (din) cudaFree(din);
  if (dout) cudaFree(dout);
  return rc;
}

// ------------------------- scan without device allocation ------------------
//
// For callers that cannot allocate device memory while they run (a host that
// hands all device memory to its own allocator at start-up and forbids any
// later cudaMalloc, or a plugin that may only use the buffers its host gives
// it).  Every intermediate array of the search lives in one file-scope device
// array of fixed size instead of memory allocated per call.
namespace {

// Largest grid: N = nz*ny*nx <= kNoAllocMaxVoxels (64^3), edges <= 256.
constexpr long long kNoAllocMaxVoxels = 64LL * 64 * 64;
constexpr int kNoAllocMaxEdge = 256;
constexpr int kNoAllocRotChunk = 1024;                       // rotations converted per chunk
constexpr size_t kNoAllocSpecBytes = 2ull * kNoAllocMaxVoxels * sizeof(float2);   // target spectra
constexpr size_t kNoAllocBufBytes = 3ull * kNoAllocMaxVoxels * sizeof(float2);    // one rotation pair
constexpr size_t kNoAllocTwBytes = 3ull * kNoAllocMaxEdge * sizeof(float2);
constexpr size_t kNoAllocRotBytes = (size_t)kNoAllocRotChunk * sizeof(RotFixed);
constexpr size_t kNoAllocBytes = kNoAllocSpecBytes + kNoAllocBufBytes + kNoAllocTwBytes + kNoAllocRotBytes;

// The scratch itself (about 10.1 MiB), held by every GPU that loads the
// library until the process exits.  Host code must not use the symbol as an
// address: the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
unsigned char* g_noalloc_addr[kNoAllocMaxDevices] = {};
size_t g_noalloc_smem[kNoAllocMaxDevices] = {};
std::mutex g_noalloc_mutex;

// One-time set-up per device, with that device current: the scratch's device
// address (cudaGetSymbolAddress), the largest shared memory a block may opt
// in to, and the kernels' dynamic shared-memory limits.  Later calls on the
// device only read what this stored.
int noalloc_setup(unsigned char** out, size_t* smem_optin) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(nullptr, PF_E_CUDA, "pf_scan_noalloc: no current CUDA device");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    int optin = 0;
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess || optin <= 0)
      return fail(nullptr, PF_E_CUDA, "pf_scan_noalloc: no shared-memory limit for device %d: %s", dev,
                  cudaGetErrorString(e));
    const size_t m = (size_t)optin;
    if ((e = allow_smem(k_pass1<false>, m)) != cudaSuccess || (e = allow_smem(k_pass2<false>, m)) != cudaSuccess ||
        (e = allow_smem(k_pass3<false>, m)) != cudaSuccess || (e = allow_smem(k_fwd_x_real, m)) != cudaSuccess)
      return fail(nullptr, PF_E_CUDA, "pf_scan_noalloc: kernel attributes: %s", cudaGetErrorString(e));
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(nullptr, PF_E_CUDA, "pf_scan_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
    g_noalloc_smem[dev] = m;
    g_noalloc_addr[dev] = (unsigned char*)ptr;
  }
  *out = g_noalloc_addr[dev];
  *smem_optin = g_noalloc_smem[dev];
  return PF_OK;
}

// The twiddle tables of the three edges, built on the device: table a (x, y,
// z) at tw + a * kNoAllocMaxEdge holds exp(-2 pi i m / n_a), m < n_a, the same
// values the contexts upload (cos and sin of the angle in float64, rounded to
// float32; sincospi takes the angle as a multiple of pi).
__global__ void k_noalloc_twiddles(float2* __restrict__ tw, int nx, int ny, int nz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * kNoAllocMaxEdge) return;
  const int a = i / kNoAllocMaxEdge, m = i - a * kNoAllocMaxEdge;
  const int n = a == 0 ? nx : (a == 1 ? ny : nz);
  if (m >= n) return;
  double sn, cs;
  sincospi(2.0 * (double)m / (double)n, &sn, &cs);
  tw[i] = make_float2((float)cs, (float)-sn);
}

__global__ void k_rot_to_fixed(const double* __restrict__ rd, long long n, RotFixed* __restrict__ out) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) {
    RotFixed f;
    for (int k = 0; k < 9; ++k) f.r[k] = llround(rd[9 * i + k] * 4294967296.0);
    out[i] = f;
  }
}

}  // namespace

int pf_scan_noalloc(int nz, int ny, int nx, const float* d_target, const uint8_t* d_lcc_mask, const float* d_tmpl,
                    const float* d_mask, double norm_factor, int rmax, const double* d_rotmats, int64_t nrot,
                    int64_t rot_offset, float* d_lcc, int32_t* d_rot, void* stream) {
  if (nz < 1 || ny < 1 || nx < 1 || nz > kNoAllocMaxEdge || ny > kNoAllocMaxEdge || nx > kNoAllocMaxEdge ||
      (long long)nz * ny * nx > kNoAllocMaxVoxels)
    return fail(nullptr, PF_E_SHAPE,
                "pf_scan_noalloc: grid (%d, %d, %d) exceeds the fixed scratch (at most %lld voxels, edges <= %d)",
                nz, ny, nx, kNoAllocMaxVoxels, kNoAllocMaxEdge);
  if (!d_target || !d_lcc_mask || !d_tmpl || !d_mask || !d_lcc || !d_rot || (!d_rotmats && nrot > 0) || nrot < 0)
    return fail(nullptr, PF_E_ARG, "pf_scan_noalloc: null pointer or negative rotation count");
  if (!(norm_factor > 0)) return fail(nullptr, PF_E_ARG, "pf_scan_noalloc: norm_factor must be positive");
  if (rmax < 0 || 2 * rmax > std::min(nz, std::min(ny, nx)))
    return fail(nullptr, PF_E_ARG, "pf_scan_noalloc: rmax %d outside [0, min(shape)//2]", rmax);
  if (rot_offset < 0 || rot_offset + nrot > (int64_t)0x7fffffff)
    return fail(nullptr, PF_E_ARG, "pf_scan_noalloc: rotation index overflows int32");
  // plans from the constexpr planner (no host allocation either)
  auto plan_of = [](int n, AxisPlan* pl) {
    const CtPlan c = ct_plan(n);
    if (c.nst < 1) return false;
    int prod = 1;
    for (int i = 0; i < c.nst; ++i) prod *= c.r[i];
    if (prod != n) return false;
    pl->n = n;
    pl->nst = c.nst;
    for (int i = 0; i < c.nst; ++i) pl->radix[i] = c.r[i];
    return true;
  };
  AxisPlan px, py, pz;
  if (!plan_of(nx, &px) || !plan_of(ny, &py) || !plan_of(nz, &pz))
    return fail(nullptr, PF_E_SHAPE, "pf_scan_noalloc: every edge must factor into 2, 3, 5 and 7");
  unsigned char* scratch = nullptr;
  size_t smem_optin = 0;
  int rc = noalloc_setup(&scratch, &smem_optin);
  if (rc) return rc;
  if (plane_smem(ny, nz) > smem_optin)
    return fail(nullptr, PF_E_SHAPE, "pf_scan_noalloc: the (z, y) plane does not fit in shared memory");
  cudaStream_t s = (cudaStream_t)stream;
  const long long N = (long long)nz * ny * nx;
  float2* spec = (float2*)scratch;
  float2* buf = (float2*)(scratch + kNoAllocSpecBytes);
  float2* twx = (float2*)(scratch + kNoAllocSpecBytes + kNoAllocBufBytes);
  float2* twy = twx + kNoAllocMaxEdge;
  float2* twz = twy + kNoAllocMaxEdge;
  RotFixed* rots = (RotFixed*)(scratch + kNoAllocSpecBytes + kNoAllocBufBytes + kNoAllocTwBytes);

  // twiddle tables, built on the device
  k_noalloc_twiddles<<<(3 * kNoAllocMaxEdge + 255) / 256, 256, 0, s>>>(twx, nx, ny, nz);
  PF_CUDA(nullptr, cudaGetLastError());

  // target spectra FT(target)/N and FT(target^2)/N into the scratch
  Geometry g{};
  g.nz = nz;
  g.ny = ny;
  g.nx = nx;
  g.rmax = rmax;
  g.reff = rmax;
  g.nvz = nz;
  g.zlo = nz - 1;
  int ty1 = 16;
  while (ty1 > 1 && ((long long)ty1 * nx > (long long)kMaxVoxPerThread * kThreadsLine || line_smem(nx, 3, ty1) > 96 * 1024))
    ty1--;
  int ty3 = 16;
  while (ty3 > 1 && (long long)ty3 * nx > (long long)kMaxVoxPerThread * kThreadsLine) ty3 /= 2;
  const long long buf_len = (long long)(kNoAllocBufBytes / sizeof(float2));
  FwdXParams fx{g, px, twx, d_target, nullptr, 1, buf, ty1, buf_len};
  k_fwd_x_real<<<dim3(nz, (ny + ty1 - 1) / ty1, 1), kThreadsLine, line_smem(nx, 3, ty1), s>>>(fx);
  PF_CUDA(nullptr, cudaGetLastError());
  Pass2Params pt{};
  pt.g = g;
  pt.py = py;
  pt.pz = pz;
  pt.twy = twy;
  pt.twz = twz;
  pt.buf = buf;
  pt.nfield = 2;
  pt.mode = 1;
  pt.out = spec;
  pt.scale = (float)(1.0 / (double)N);
  pt.buf_len = buf_len;
  pt.out_len = 2 * N;
  k_pass2<false><<<dim3(nx, 2, 1), kThreadsPlane, plane_smem(ny, nz), s>>>(pt);
  PF_CUDA(nullptr, cudaGetLastError());

  // the outputs start at zero (strict > against 0, rotation 0)
  PF_CUDA(nullptr, cudaMemsetAsync(d_lcc, 0, N * sizeof(float), s));
  PF_CUDA(nullptr, cudaMemsetAsync(d_rot, 0, N * sizeof(int32_t), s));

  // one rotation pair per pass: buf holds exactly one pair
  for (int64_t c0 = 0; c0 < nrot; c0 += kNoAllocRotChunk) {
    const int64_t cn = std::min<int64_t>(kNoAllocRotChunk, nrot - c0);
    k_rot_to_fixed<<<(unsigned)((cn + 127) / 128), 128, 0, s>>>(d_rotmats + 9 * c0, cn, rots);
    PF_CUDA(nullptr, cudaGetLastError());
    for (int64_t r0 = 0; r0 < cn; r0 += 2) {
      Pass1Params p1{g, px, GatherSrc{d_tmpl, d_mask}, twx, rots, d_rotmats + 9 * c0, r0, cn, buf, ty1, nullptr, 0,
                     buf_len};
      k_pass1<false><<<dim3(nz, (ny + ty1 - 1) / ty1, 1), kThreadsLine, line_smem(nx, 3, ty1), s>>>(p1);
      Pass2Params p2{};
      p2.g = g;
      p2.py = py;
      p2.pz = pz;
      p2.twy = twy;
      p2.twz = twz;
      p2.buf = buf;
      p2.s1 = spec;
      p2.s2 = spec + N;
      p2.nfield = 3;
      p2.mode = 0;
      p2.buf_len = buf_len;
      p2.spec_len = N;
      k_pass2<false><<<dim3(nx, 3, 1), kThreadsPlane, plane_smem(ny, nz), s>>>(p2);
      Pass3Params p3{g, px, twx, buf, 1, r0, cn, rot_offset + c0, d_lcc_mask, (float)norm_factor,
                     d_lcc, d_rot, ty3, 0};
      p3.buf_len = buf_len;
      k_pass3<false><<<dim3(nz, (ny + ty3 - 1) / ty3, 1), kThreadsLine, line_smem(nx, 3, ty3), s>>>(p3);
      PF_CUDA(nullptr, cudaGetLastError());
    }
  }
  return PF_OK;
}

// ----------------------------- unit-level mirrors ---------------------------

int pf_rotate_grid3d(const double* grid, int nz, int ny, int nx, const double* rotmat, int radius, double* out,
                     int nearest) {
  if (!grid || !rotmat || !out || nz < 1 || ny < 1 || nx < 1 || radius < 0)
    return fail(nullptr, PF_E_ARG, "pf_rotate_grid3d: bad arguments");
  if (radius >= std::min(nz, std::min(ny, nx)))
    return fail(nullptr, PF_E_ARG, "radius %d must be smaller than every grid edge", radius);
  const long long N = (long long)nz * ny * nx;
  float* dg = nullptr;
  double *dout = nullptr, *drd = nullptr;
  int rc = alloc(nullptr, (void**)&dg, N * sizeof(float));
  if (!rc) rc = alloc(nullptr, (void**)&dout, N * sizeof(double));
  if (!rc) rc = alloc(nullptr, (void**)&drd, 9 * sizeof(double));
  std::vector<float> hg;
  if (!rc) {
    hg.resize((size_t)N);
    for (long long i = 0; i < N; ++i) hg[i] = (float)grid[i];
    if (cudaMemcpy(dg, hg.data(), N * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dout, out, N * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(drd, rotmat, 9 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      rc = fail(nullptr, PF_E_CUDA, "upload failed");
  }
  if (!rc) {
    Geometry g{};
    g.nz = nz;
    g.ny = ny;
    g.nx = nx;
    g.rmax = radius;
    g.reff = radius;
    GatherSrc src{dg, dg};
    k_rotate_grid<<<(unsigned)std::min<long long>((N + 255) / 256, 4096), 256>>>(g, src, to_fixed(rotmat), drd,
                                                                                radius, nearest, dout);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = fail(nullptr, PF_E_CUDA, "rotate kernel: %s", cudaGetErrorString(e));
  }
  if (!rc && cudaMemcpy(out, dout, N * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = fail(nullptr, PF_E_CUDA, "download failed");
  if (dg) cudaFree(dg);
  if (dout) cudaFree(dout);
  if (drd) cudaFree(drd);
  return rc;
}

int pf_conj_multiply(const double* in1, const double* in2, double* out, int64_t n) {
  if (!in1 || !in2 || !out || n < 0) return fail(nullptr, PF_E_ARG, "pf_conj_multiply: bad arguments");
  if (n == 0) return PF_OK;
  double2 *a = nullptr, *b = nullptr, *o = nullptr;
  int rc = alloc(nullptr, (void**)&a, n * sizeof(double2));
  if (!rc) rc = alloc(nullptr, (void**)&b, n * sizeof(double2));
  if (!rc) rc = alloc(nullptr, (void**)&o, n * sizeof(double2));
  if (!rc && (cudaMemcpy(a, in1, n * sizeof(double2), cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(b, in2, n * sizeof(double2), cudaMemcpyHostToDevice) != cudaSuccess))
    rc = fail(nullptr, PF_E_CUDA, "upload failed");
  if (!rc) {
    k_conj_multiply<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256>>>(a, b, o, n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, o, n * sizeof(double2), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = fail(nullptr, PF_E_CUDA, "conj_multiply: %s", cudaGetErrorString(e));
  }
  if (a) cudaFree(a);
  if (b) cudaFree(b);
  if (o) cudaFree(o);
  return rc;
}

int pf_calc_lcc(const double* gcc, const double* ave, const double* ave2, const uint8_t* mask, double* lcc,
                int64_t n) {
  if (!gcc || !ave || !ave2 || !mask || !lcc || n < 0) return fail(nullptr, PF_E_ARG, "pf_calc_lcc: bad arguments");
  if (n == 0) return PF_OK;
  double *dg = nullptr, *da = nullptr, *da2 = nullptr, *dl = nullptr;
  unsigned char* dm = nullptr;
  int rc = alloc(nullptr, (void**)&dg, n * sizeof(double));
  if (!rc) rc = alloc(nullptr, (void**)&da, n * sizeof(double));
  if (!rc) rc = alloc(nullptr, (void**)&da2, n * sizeof(double));
  if (!rc) rc = alloc(nullptr, (void**)&dl, n * sizeof(double));
  if (!rc) rc = alloc(nullptr, (void**)&dm, n);
  if (!rc && (cudaMemcpy(dg, gcc, n * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(da, ave, n * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(da2, ave2, n * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(dl, lcc, n * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(dm, mask, n, cudaMemcpyHostToDevice) != cudaSuccess))
    rc = fail(nullptr, PF_E_CUDA, "upload failed");
  if (!rc) {
    k_calc_lcc<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256>>>(dg, da, da2, dm, dl, n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(lcc, dl, n * 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = fail(nullptr, PF_E_CUDA, "calc_lcc: %s", cudaGetErrorString(e));
  }
  void* ptrs[] = {dg, da, da2, dl, dm};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  return rc;
}

int pf_combine(float* lcc, int32_t* rot, const float* part_lcc, const int32_t* part_rot, int64_t n, int64_t rot_add) {
  if (!lcc || !rot || !part_lcc || !part_rot || n < 0) return fail(nullptr, PF_E_ARG, "pf_combine: bad arguments");
  if (n == 0) return PF_OK;
  float *dl = nullptr, *dpl = nullptr;
  int *dr = nullptr, *dpr = nullptr;
  int rc = alloc(nullptr, (void**)&dl, n * 4);
  if (!rc) rc = alloc(nullptr, (void**)&dpl, n * 4);
  if (!rc) rc = alloc(nullptr, (void**)&dr, n * 4);
  if (!rc) rc = alloc(nullptr, (void**)&dpr, n * 4);
  if (!rc && (cudaMemcpy(dl, lcc, n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(dpl, part_lcc, n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(dr, rot, n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(dpr, part_rot, n * 4, cudaMemcpyHostToDevice) != cudaSuccess))
    rc = fail(nullptr, PF_E_CUDA, "upload failed");
  if (!rc) {
    k_combine<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256>>>(dpl, dpr, rot_add, dl, dr, n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(lcc, dl, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(rot, dr, n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = fail(nullptr, PF_E_CUDA, "combine: %s", cudaGetErrorString(e));
  }
  void* ptrs[] = {dl, dpl, dr, dpr};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  return rc;
}

}  // extern "C"
