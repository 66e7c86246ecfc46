// Split-bf16x3 tensor-core DFT stages (precision-study variant, sm_103a).
//
// A radix-R Stockham stage (R <= 16) as a matrix product on the tensor cores:
// the R-point DFT of one butterfly is y = F x with F[m][k] = W_R^{mk}, in real
// form
//     [yr]   [Fr  -Fi] [xr]
//     [yi] = [Fi   Fr] [xi]          (32 x 32, zero beyond R)
// and eight butterflies of a warp are the eight columns of one
// mma.sync.m16n8k16 bf16 tile set (2 x 2 tiles of 16 x 16).  Every float32
// operand is split into two bfloat16 parts, v = hi + lo (hi = bf16(v),
// lo = bf16(v - hi)), and a product is accumulated in float32 as
//     A.B ~ A_lo.B_hi + A_hi.B_lo + A_hi.B_hi
// (the split-bf16x3 scheme; the lo.lo term is dropped).  Twiddles between
// stages stay float32 multiplies, as in the float32 engine.
//
// Same stage contract as fft_stage (pf_fft.cuh): items (line, j) in chunks of
// lines, every item of a chunk loaded before any is stored when src and dst
// alias, one barrier on each side.
#pragma once
#include <cuda_bf16.h>

#include "pf_fft.cuh"

namespace pf {

constexpr int kMmaGroups = 4;   // groups of 8 butterflies a warp holds per chunk

__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

// two bf16 in one register: `first` in the low half (the lower row/column index)
__device__ __forceinline__ unsigned int pack2(__nv_bfloat16 first, __nv_bfloat16 second) {
  return (unsigned int)__bfloat16_as_ushort(first) | ((unsigned int)__bfloat16_as_ushort(second) << 16);
}

// d += a (16x16, row major) * b (16x8, column major); bf16 in, float32 accumulate
__device__ __forceinline__ void mma_16816(float (&d)[4], const unsigned int (&a)[4], unsigned int b0, unsigned int b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// The lane's fragments of the four 16x16 tiles of the real DFT matrix, split:
// tile (mt, kt): (0,0) = Fr, (0,1) = -Fi, (1,0) = Fi, (1,1) = Fr.
struct DftFragments {
  unsigned int fr_hi[4], fr_lo[4], fi_hi[4], fi_lo[4], nfi_hi[4], nfi_lo[4];
};

// Lane (g = lane/4, t = lane%4) holds rows m in {g, g+8} and columns
// k in {2t, 2t+1, 2t+8, 2t+9} of each tile (register q: rows g + 8*(q&1),
// columns 2t + 8*(q>>1) + {0, 1}).  W_R^e = tw[(e mod R) * L/R] (forward
// values of a length-L table); the inverse conjugates.
template <bool INV>
__device__ __forceinline__ DftFragments dft_fragments(int R, int L, const float2* __restrict__ tw) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int step = L / R;
  DftFragments f;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int m = g + 8 * (q & 1);
    __nv_bfloat16 rh[2], rl[2], ih[2], il[2], nh[2], nl[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int k = 2 * t + 8 * (q >> 1) + e;
      float wr = 0.f, wi = 0.f;
      if (m < R && k < R) {
        const float2 w = tw[((m * k) % R) * step];
        wr = w.x;
        wi = INV ? -w.y : w.y;
      }
      split_bf16(wr, rh[e], rl[e]);
      split_bf16(wi, ih[e], il[e]);
      split_bf16(-wi, nh[e], nl[e]);
    }
    f.fr_hi[q] = pack2(rh[0], rh[1]);
    f.fr_lo[q] = pack2(rl[0], rl[1]);
    f.fi_hi[q] = pack2(ih[0], ih[1]);
    f.fi_lo[q] = pack2(il[0], il[1]);
    f.nfi_hi[q] = pack2(nh[0], nh[1]);
    f.nfi_lo[q] = pack2(nl[0], nl[1]);
  }
  return f;
}

// d += A.B in split-bf16x3 (small terms first)
__device__ __forceinline__ void mma_split3(float (&d)[4], const unsigned int (&a_hi)[4], const unsigned int (&a_lo)[4],
                                           const unsigned int (&b_hi)[2], const unsigned int (&b_lo)[2]) {
  mma_16816(d, a_lo, b_hi[0], b_hi[1]);
  mma_16816(d, a_hi, b_lo[0], b_lo[1]);
  mma_16816(d, a_hi, b_hi[0], b_hi[1]);
}

// One radix-R stage (2 <= R <= 16) of `nlines` lines of length L, as fft_stage.
template <bool INV, class Src, class Dst>
__device__ __noinline__ void fft_stage_mma(int R, int nlines, int L, int Ns, const float2* __restrict__ tw,
                                           const Src src, const Dst dst, bool alias) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int nb = L / R;
  const int twmul = L / (Ns * R);
  const DftFragments F = dft_fragments<INV>(R, L, tw);
  // lines per chunk: every warp holds at most kMmaGroups groups of 8 items
  int C = (8 * kMmaGroups * nwarps) / nb;
  if (C > nlines) C = nlines;
  if (C < 1) C = 1;  // the host limits edges so that one line always fits
  for (int l0 = 0; l0 < nlines; l0 += C) {
    const int cl = min(C, nlines - l0);
    const int items = cl * nb;
    float yr[kMmaGroups][4], yi[kMmaGroups][4];
#pragma unroll
    for (int q = 0; q < kMmaGroups; ++q) {
      const int group = warp + q * nwarps;
      // B operand: item n = g of the group, inputs k in {2t, 2t+1, 2t+8, 2t+9}
      const int it = group * 8 + g;
      float xr[4] = {0.f, 0.f, 0.f, 0.f}, xi[4] = {0.f, 0.f, 0.f, 0.f};
      if (it < items) {
        const int line = l0 + it % cl;
        const int j = it / cl;
        const int jm = (j % Ns) * twmul;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          const int r = 2 * t + (s & 1) + 8 * (s >> 1);
          if (r < R) {
            float2 v = src.load(line, j + r * nb);
            if (r > 0 && Ns > 1) {
              float2 w = PF_CHECK(kChkTwiddle, r * jm, L) ? tw[r * jm] : make_float2(1.f, 0.f);
              if (INV) w.y = -w.y;
              v = cmul(v, w);
            }
            xr[s] = v.x;
            xi[s] = v.y;
          }
        }
      }
      unsigned int br_hi[2], br_lo[2], bi_hi[2], bi_lo[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        __nv_bfloat16 a0, a1, b0, b1, c0, c1, d0, d1;
        split_bf16(xr[2 * h], a0, b0);
        split_bf16(xr[2 * h + 1], a1, b1);
        split_bf16(xi[2 * h], c0, d0);
        split_bf16(xi[2 * h + 1], c1, d1);
        br_hi[h] = pack2(a0, a1);
        br_lo[h] = pack2(b0, b1);
        bi_hi[h] = pack2(c0, c1);
        bi_lo[h] = pack2(d0, d1);
      }
      // yr = Fr xr - Fi xi ; yi = Fi xr + Fr xi  (the whole warp takes part, valid items or not)
#pragma unroll
      for (int e = 0; e < 4; ++e) yr[q][e] = yi[q][e] = 0.f;
      mma_split3(yr[q], F.nfi_hi, F.nfi_lo, bi_hi, bi_lo);
      mma_split3(yr[q], F.fr_hi, F.fr_lo, br_hi, br_lo);
      mma_split3(yi[q], F.fr_hi, F.fr_lo, bi_hi, bi_lo);
      mma_split3(yi[q], F.fi_hi, F.fi_lo, br_hi, br_lo);
    }
    if (alias) __syncthreads();
#pragma unroll
    for (int q = 0; q < kMmaGroups; ++q) {
      const int group = warp + q * nwarps;
      // D: outputs m in {g, g+8} of items n in {2t, 2t+1}
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int it = group * 8 + 2 * t + e;
        if (it < items) {
          const int line = l0 + it % cl;
          const int j = it / cl;
          const int base = (j / Ns) * Ns * R + (j % Ns);
          if (g < R) dst.store(line, base + g * Ns, make_float2(yr[q][e], yi[q][e]));
          if (g + 8 < R) dst.store(line, base + (g + 8) * Ns, make_float2(yr[q][2 + e], yi[q][2 + e]));
        }
      }
    }
    if (alias) __syncthreads();
  }
}

}  // namespace pf
