// Split-bf16x3 DFT stages on the fifth-generation tensor cores (tcgen05),
// a precision-study variant of the plane pass (sm_103a).
//
// A radix-R Stockham stage (2 <= R <= 16) of up to 512 items (line, j) at a
// time: the R-point DFTs of 128 items are one matrix product
//
//     D[m][n] = sum_k A[m][k] B[n][k]          (M = 128, N = 32, K = 32)
//
// with row m of A the item's twiddled inputs in real form (k < 16: real
// parts x_r, k >= 16: imaginary parts, zero beyond R) and B the DFT matrix
// in real block form (n < 16: Re y_n = sum Fr x_r - Fi x_i, n >= 16:
// Im y_{n-16} = sum Fi x_r + Fr x_i).  Every float32 operand is split into
// bfloat16 hi + lo parts and D = A_lo B_hi + A_hi B_lo + A_hi B_hi is
// accumulated in float32 in tensor memory (the lo.lo term dropped, as in the
// mma.sync variant of pf_fft_mma.cuh).
//
// Per chunk: every thread writes its item's A rows (hi and lo) into shared
// memory in the canonical K-major layout without swizzle (core matrices of
// 8 rows x 16 bytes; the K-adjacent core matrices 128 B apart (leading byte
// offset), the 8-row groups 512 B apart (stride byte offset)); one thread
// issues the 24 MMAs of the four 128-item tiles (tcgen05.mma, kind::f16,
// operands by shared-memory descriptors, accumulators in 4 x 32 tensor-memory
// columns) and commits them to an mbarrier; every thread waits on it
// (bounded), reads its item's 32 accumulators from its own tensor-memory lane
// (tcgen05.ld 32x32b) and stores the R outputs in Stockham order.
//
// The block allocates 128 tensor-memory columns once (tc05_begin) and frees
// them before it exits (tc05_end).  A wait that runs out (2 s on the global
// timer) records an error in g_tc05_error; the block then skips its remaining
// chunks, waits once more (bounded) for the products in flight and frees the
// tensor memory, so the search returns an error instead of hanging.
#pragma once
#include <cuda_bf16.h>

#include "pf_fft.cuh"

namespace pf {

constexpr int kTc05Threads = 512;                  // block size of the plane pass that uses it
constexpr int kTc05Tiles = kTc05Threads / 128;     // 128-item tiles per chunk
constexpr int kTc05Cols = 32 * kTc05Tiles;         // tensor-memory columns (a power of two >= 32)
constexpr int kTc05TileBytes = 128 * 32 * 2;       // one bf16 A tile (M = 128, K = 32)
constexpr int kTc05BBytes = 32 * 32 * 2;           // one bf16 B matrix (N = 32, K = 32)
// shared memory of the operands: A hi + lo of every tile, B hi + lo
constexpr int kTc05SmemBytes = 2 * kTc05Tiles * kTc05TileBytes + 2 * kTc05BBytes;
constexpr unsigned long long kTc05WaitNs = 2000000000ull;  // a wait gives up after 2 s

// per-block state of the tcgen05 stages
struct Tc05State {
  unsigned long long mbar;    // MMA completion barrier
  unsigned int tmem;          // tensor-memory address of the 128 allocated columns
  unsigned int phase;         // parity of the next completion
  unsigned int ops;           // shared-memory address of the operand area (1024-aligned)
  int failed;                 // a wait ran out in this block
};

__device__ __forceinline__ Tc05State& tc05_state() {
  __shared__ Tc05State st;
  return st;
}

// nonzero after a wait ran out (read and cleared by the host)
__device__ int g_tc05_error;

// byte offset of element (m, k) in a K-major no-swizzle bf16 tile of 32 K-columns
__host__ __device__ constexpr int tc05_off(int m, int k) {
  return (m >> 3) * 512 + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2;
}

// shared-memory matrix descriptor: start address, leading byte offset 128
// (K-adjacent core matrices), stride byte offset 512 (8-row groups), no swizzle
__device__ __forceinline__ unsigned long long tc05_desc(unsigned int saddr) {
  return (unsigned long long)((saddr & 0x3FFFF) >> 4) | ((unsigned long long)(128 >> 4) << 16) |
         ((unsigned long long)(512 >> 4) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: float32 D, bf16 A and B, both K-major, N = 32, M = 128
constexpr unsigned int kTc05Idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ unsigned int smem_u32(const void* p) {
  return (unsigned int)__cvta_generic_to_shared(p);
}

// Allocate the tensor memory and set up the barrier; every thread of the block
// calls it once, before the first stage.  `ops`: the operand area, 1024-aligned.
__device__ __forceinline__ void tc05_begin(void* ops) {
  Tc05State& st = tc05_state();
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&st.tmem)),
                 "n"(kTc05Cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&st.mbar)) : "memory");
    st.phase = 0;
    st.ops = smem_u32(ops);
    st.failed = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ bool tc05_wait(unsigned int mbar, unsigned int parity);

// Free the tensor memory (every thread calls it once, after the last stage).
// After a wait ran out, first wait once more (bounded) for the products in
// flight, so that no MMA writes columns that are already freed.
__device__ __forceinline__ void tc05_end() {
  Tc05State& st = tc05_state();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (st.failed) tc05_wait(smem_u32(&st.mbar), st.phase);
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(st.tmem), "n"(kTc05Cols) : "memory");
  if (threadIdx.x == 0 && st.failed) atomicExch(&g_tc05_error, 1);
}

__device__ __forceinline__ unsigned int tc05_pack(float a, float b, unsigned int& lo_pair) {
  const __nv_bfloat16 ha = __float2bfloat16_rn(a), hb = __float2bfloat16_rn(b);
  const __nv_bfloat16 la = __float2bfloat16_rn(a - __bfloat162float(ha));
  const __nv_bfloat16 lb = __float2bfloat16_rn(b - __bfloat162float(hb));
  lo_pair = (unsigned int)__bfloat16_as_ushort(la) | ((unsigned int)__bfloat16_as_ushort(lb) << 16);
  return (unsigned int)__bfloat16_as_ushort(ha) | ((unsigned int)__bfloat16_as_ushort(hb) << 16);
}

// Write 32 float32 values of row m of a K-major tile as bf16 hi (at `hi`) and
// lo (at `lo`): four 16-byte stores each.
__device__ __forceinline__ void tc05_write_row(unsigned int hi, unsigned int lo, int m, const float (&v)[32]) {
#pragma unroll
  for (int kc = 0; kc < 4; ++kc) {
    unsigned int h[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) h[e] = tc05_pack(v[8 * kc + 2 * e], v[8 * kc + 2 * e + 1], l[e]);
    const unsigned int off = (unsigned int)tc05_off(m, 8 * kc);
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(hi + off), "r"(h[0]), "r"(h[1]), "r"(h[2]),
                 "r"(h[3])
                 : "memory");
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(lo + off), "r"(l[0]), "r"(l[1]), "r"(l[2]),
                 "r"(l[3])
                 : "memory");
  }
}

__device__ __forceinline__ void tc05_mma(unsigned int d, unsigned long long a, unsigned long long b, int acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(kTc05Idesc), "r"(acc)
      : "memory");
}

// Bounded wait for completion `parity` of the barrier; false if it ran out.
// Non-blocking tests against the global nanosecond timer, about two seconds
// at most (mbarrier.try_wait may suspend the thread for a system-dependent
// time per call, so a count of calls bounds nothing).
__device__ __forceinline__ unsigned long long tc05_now() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool tc05_wait(unsigned int mbar, unsigned int parity) {
  const unsigned long long t0 = tc05_now();
  for (;;) {
    unsigned int done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    if (tc05_now() - t0 > kTc05WaitNs) return false;
  }
}

// One radix-R stage (2 <= R <= 16) of `nlines` lines of length L (the
// contract of fft_stage); blockDim.x == kTc05Threads, between tc05_begin and
// tc05_end.
template <bool INV, class Src, class Dst>
__device__ __noinline__ void fft_stage_tc05(int R, int nlines, int L, int Ns, const float2* __restrict__ tw,
                                            const Src src, const Dst dst, bool alias) {
  Tc05State& st = tc05_state();
  const int t = threadIdx.x;
  const int nb = L / R;
  const int twmul = L / (Ns * R);
  const unsigned int a_hi = st.ops, a_lo = st.ops + kTc05Tiles * kTc05TileBytes;
  const unsigned int b_hi = st.ops + 2 * kTc05Tiles * kTc05TileBytes, b_lo = b_hi + kTc05BBytes;
  // the DFT matrix of this stage in real block form: thread n < 32 writes row n
  if (t < 32) {
    const int n = t & 15;
    const bool im = t >= 16;
    float v[32];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      float fr = 0.f, fi = 0.f;
      if (n < R && r < R) {
        const float2 w = tw[((n * r) % R) * (L / R)];
        fr = w.x;
        fi = INV ? -w.y : w.y;
      }
      v[r] = im ? fi : fr;          // Re: Fr x_r ; Im: Fi x_r
      v[16 + r] = im ? fr : -fi;    // Re: -Fi x_i ; Im: Fr x_i
    }
    tc05_write_row(b_hi, b_lo, t, v);
  }
  int cl = kTc05Threads / nb;
  if (cl > nlines) cl = nlines;
  if (cl < 1) cl = 1;   // nb <= 128 < 512 on every planned edge
  const int q = t >> 7, m = t & 127;
  for (int l0 = 0; l0 < nlines; l0 += cl) {
    if (st.failed) break;                  // uniform: read after a block barrier
    const int cn = min(cl, nlines - l0);
    const int items = cn * nb;
    const bool mine = t < items;
    const int line = l0 + t % cn;
    const int j = t / cn;
    {
      float v[32];
#pragma unroll
      for (int r = 0; r < 16; ++r) { v[r] = 0.f; v[16 + r] = 0.f; }
      if (mine) {
        const int jm = (j % Ns) * twmul;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
          if (r < R) {
            float2 x = src.load(line, j + r * nb);
            if (r > 0 && Ns > 1) {
              float2 w = PF_CHECK(kChkTwiddle, r * jm, L) ? tw[r * jm] : make_float2(1.f, 0.f);
              if (INV) w.y = -w.y;
              x = cmul(x, w);
            }
            v[r] = x.x;
            v[16 + r] = x.y;
          }
        }
      }
      tc05_write_row(a_hi + q * kTc05TileBytes, a_lo + q * kTc05TileBytes, m, v);
    }
    // the operands are visible to the tensor cores; one thread issues the products
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    const unsigned int parity = st.phase;
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const unsigned long long bh0 = tc05_desc(b_hi), bh1 = tc05_desc(b_hi + 256);
      const unsigned long long bl0 = tc05_desc(b_lo), bl1 = tc05_desc(b_lo + 256);
#pragma unroll
      for (int tile = 0; tile < kTc05Tiles; ++tile) {
        const unsigned int d = st.tmem + 32 * tile;
        const unsigned int ah = a_hi + tile * kTc05TileBytes, al = a_lo + tile * kTc05TileBytes;
        tc05_mma(d, tc05_desc(al), bh0, 0);          // A_lo B_hi (K 0..15)
        tc05_mma(d, tc05_desc(al + 256), bh1, 1);    //            (K 16..31)
        tc05_mma(d, tc05_desc(ah), bl0, 1);          // A_hi B_lo
        tc05_mma(d, tc05_desc(ah + 256), bl1, 1);
        tc05_mma(d, tc05_desc(ah), bh0, 1);          // A_hi B_hi
        tc05_mma(d, tc05_desc(ah + 256), bh1, 1);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&st.mbar))
                   : "memory");
    }
    const bool ok = tc05_wait(smem_u32(&st.mbar), parity);
    if (!ok) st.failed = 1;                // seen by every thread after the next barrier
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // this thread's item: lane m of its warp's quadrant, columns 32 q .. 32 q + 31
    unsigned int d[32];
    const unsigned int taddr = st.tmem + ((unsigned int)(32 * ((t >> 5) & 3)) << 16) + 32 * q;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]),
          "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]), "=r"(d[14]), "=r"(d[15]),
          "=r"(d[16]), "=r"(d[17]), "=r"(d[18]), "=r"(d[19]), "=r"(d[20]), "=r"(d[21]), "=r"(d[22]), "=r"(d[23]),
          "=r"(d[24]), "=r"(d[25]), "=r"(d[26]), "=r"(d[27]), "=r"(d[28]), "=r"(d[29]), "=r"(d[30]), "=r"(d[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();                       // every input read and every accumulator loaded
    if (t == 0 && !st.failed) st.phase = parity ^ 1u;
    if (mine) {
      const int base = (j / Ns) * Ns * R + (j % Ns);
#pragma unroll
      for (int r = 0; r < 16; ++r)
        if (r < R) dst.store(line, base + r * Ns, make_float2(__uint_as_float(d[r]), __uint_as_float(d[16 + r])));
    }
    __syncthreads();                       // stores done before the next chunk (or stage) reads
  }
  (void)alias;
}

}  // namespace pf
