// Bounds checks of the search kernels' memory accesses (debug build).
//
// Built with -DPF_BOUNDS_CHECK, every access of the search kernels to global,
// shared or distributed shared memory first checks its index against the
// extent of the array it addresses.  An index outside records the violation
// in a device word (the first violation's site and index, and a count) and
// the access is skipped -- a load reads zero, a store does nothing -- so that
// the kernel runs on without touching memory it does not own, and no check
// ever traps.  pf_debug_bounds() reads the words back.
//
// Without PF_BOUNDS_CHECK every check is the constant `true` and compiles away.
#pragma once
#include <cuda_runtime.h>

namespace pf {

// Sites of the checks (the top 16 bits of a recorded violation).
enum CheckSite : int {
  kChkTwiddle = 1,    // twiddle table of a transform
  kChkSmem = 2,       // element of a shared-memory array
  kChkGather = 3,     // template / mask voxel of the rotation gather
  kChkRowList = 4,    // pass-1 row list entry or tile row
  kChkBufStore = 5,   // store to the intermediate spectra
  kChkBufLoad = 6,    // load from the intermediate spectra
  kChkSpectrum = 7,   // target spectrum operand of the product
  kChkOut = 8,        // output spectra of a forward-only plane pass
  kChkCluster = 9,    // push into another block of the cluster
  kChkVoxel = 10,     // voxel of the lcc / rot / lcc-mask / input arrays
  kChkVoxelList = 11, // pass-3 list of the voxels inside the lcc mask
  kChkRotation = 12,  // per-rotation maximum
};

#ifdef PF_BOUNDS_CHECK

struct CheckWord {
  unsigned long long first;   // (site << 48) | (index & (2^48 - 1)) of the first violation; 0: none
  unsigned long long count;   // violations since the last read
};

// one word per translation unit (device code of separate units is not linked)
static __device__ CheckWord g_check_word;

static __device__ __noinline__ void check_failed(int site, long long index) {
  atomicAdd(&g_check_word.count, 1ull);
  const unsigned long long code =
      ((unsigned long long)(unsigned int)site << 48) | ((unsigned long long)index & 0xffffffffffffull);
  atomicCAS(&g_check_word.first, 0ull, code);
}

// index in [0, n)
__device__ __forceinline__ bool check_index(int site, long long index, long long n) {
  if (index >= 0 && index < n) return true;
  check_failed(site, index);
  return false;
}

extern __shared__ float2 g_check_dyn_smem[];   // starts where every kernel's dynamic shared memory starts

// `bytes` at `p` inside the launch's dynamic shared memory
__device__ __forceinline__ bool check_smem(int site, const void* p, int bytes) {
  unsigned int size;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(size));
  const long long off = (long long)((const char*)p - (const char*)g_check_dyn_smem);
  return check_index(site, off, (long long)size - bytes + 1);
}

#define PF_CHECK(site, index, n) ::pf::check_index((site), (long long)(index), (long long)(n))
#define PF_CHECK_SMEM(site, ptr, bytes) ::pf::check_smem((site), (ptr), (bytes))

#else

// (the operands are named, not evaluated, so that a value used only in checks is not "unused")
#define PF_CHECK(site, index, n) ((void)sizeof(index), (void)sizeof(n), true)
#define PF_CHECK_SMEM(site, ptr, bytes) ((void)sizeof(ptr), true)

#endif  // PF_BOUNDS_CHECK

}  // namespace pf

#ifdef PF_BOUNDS_CHECK
// Host side: every translation unit registers a reader of its word (defined
// in pf_api.cu), which pf_debug_bounds() calls on the current device.
int pf_check_register(int (*take)(unsigned long long* first, unsigned long long* count));

namespace {
int check_take_unit(unsigned long long* first, unsigned long long* count) {
  pf::CheckWord w{};
  if (cudaMemcpyFromSymbol(&w, pf::g_check_word, sizeof(w)) != cudaSuccess) return -1;
  const pf::CheckWord zero{};
  if (cudaMemcpyToSymbol(pf::g_check_word, &zero, sizeof(zero)) != cudaSuccess) return -1;
  *first = w.first;
  *count = w.count;
  return 0;
}
const int g_check_registered = pf_check_register(&check_take_unit);
}  // namespace
#endif
