// Shared-memory mixed-radix FFT engine for the LCC search (sm_103a).
//
// Transforms are batches of complex float32 lines held in shared memory (or
// produced/consumed by caller functors).  Each radix-R stage is a Stockham
// autosort step: load x[line][j + r*L/R], twiddle by W_{Ns*R}^{r*(j mod Ns)},
// R-point DFT in registers, store y[line][(j/Ns)*Ns*R + (j mod Ns) + r*Ns].
// The R-point DFTs are compile-time codelets (radix 2, 3, 5, 7 directly,
// composite radices by in-register Cooley-Tukey with constant twiddles).
//
// Forward transforms use W = exp(-2 pi i / n); inverse ones exp(+2 pi i / n)
// and are not normalised (the 1/N of the inverse is folded into the target
// spectra by the caller).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pf_check.cuh"

namespace pf {

// ---------------------------------------------------------------------------
// compile-time trigonometry (Taylor series in double, evaluated by the compiler)
// ---------------------------------------------------------------------------
constexpr double kPi = 3.14159265358979323846264338327950288;

__host__ __device__ constexpr double ct_sin(double x) {
  double term = x, sum = x;
  for (int k = 1; k < 40; ++k) { term *= -x * x / ((2.0 * k) * (2.0 * k + 1.0)); sum += term; }
  return sum;
}
__host__ __device__ constexpr double ct_cos(double x) {
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 40; ++k) { term *= -x * x / ((2.0 * k - 1.0) * (2.0 * k)); sum += term; }
  return sum;
}
// real and imaginary parts of exp(-+ 2 pi i m / n) (forward: minus)
__host__ __device__ constexpr double ct_twr(int m, int n) {
  m = ((m % n) + n) % n;
  if (m == 0) return 1.0;
  if (2 * m == n) return -1.0;
  if (4 * m == n || 4 * m == 3 * n) return 0.0;
  double a = 2.0 * kPi * m / n;
  if (a > kPi) a -= 2.0 * kPi;
  return ct_cos(a);
}
__host__ __device__ constexpr double ct_twi(int m, int n, bool inv) {
  m = ((m % n) + n) % n;
  double s = 0.0;
  if (m == 0 || 2 * m == n) s = 0.0;
  else if (4 * m == n) s = 1.0;
  else if (4 * m == 3 * n) s = -1.0;
  else {
    double a = 2.0 * kPi * m / n;
    if (a > kPi) a -= 2.0 * kPi;
    s = ct_sin(a);
  }
  return inv ? s : -s;
}

// Complex add / subtract.  With PF_PACKED_F32X2 (the default) they use the
// packed two-lane FP32 instructions of sm_100+ (add/sub.rn.f32x2): one issue
// slot per complex add instead of two, the same rounding as two scalar adds.
#ifndef PF_PACKED_F32X2
#define PF_PACKED_F32X2 1
#endif

#if PF_PACKED_F32X2
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  float2 d;
  asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
      " add.rn.f32x2 rd, ra, rb;\n mov.b64 {%0, %1}, rd;\n}\n"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  float2 d;
  asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
      " sub.rn.f32x2 rd, ra, rb;\n mov.b64 {%0, %1}, rd;\n}\n"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
// a + b * (s0, s1) per lane (fused multiply-add, packed)
__device__ __forceinline__ float2 cfma_lanes(float2 b, float s0, float s1, float2 a) {
  float2 d;
  asm("{\n .reg .b64 ra, rb, rs, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
      " mov.b64 rs, {%6, %7};\n fma.rn.f32x2 rd, rb, rs, ra;\n mov.b64 {%0, %1}, rd;\n}\n"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(s0), "f"(s1));
  return d;
}
#else
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cfma_lanes(float2 b, float s0, float s1, float2 a) {
  return make_float2(fmaf(b.x, s0, a.x), fmaf(b.y, s1, a.y));
}
#endif
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // conj(a) * b
  return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// multiply by the constant twiddle W_N^M (exact for multiples of quarter turns)
template <int M, int N, bool INV>
__device__ __forceinline__ float2 twc(float2 v) {
  constexpr int m = ((M % N) + N) % N;
  if constexpr (m == 0) {
    return v;
  } else if constexpr (2 * m == N) {
    return make_float2(-v.x, -v.y);
  } else if constexpr (4 * m == N) {          // forward: -i, inverse: +i
    return INV ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
  } else if constexpr (4 * m == 3 * N) {      // forward: +i, inverse: -i
    return INV ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
  } else {
    constexpr float c = (float)ct_twr(m, N);
    constexpr float s = (float)ct_twi(m, N, INV);
    return make_float2(v.x * c - v.y * s, v.x * s + v.y * c);
  }
}

// ---------------------------------------------------------------------------
// R-point DFT codelets on v[0..R-1] (natural order in and out)
// ---------------------------------------------------------------------------
template <int R, bool INV> struct DFT;

template <bool INV> struct DFT<1, INV> {
  __device__ __forceinline__ static void run(float2*) {}
};

template <bool INV> struct DFT<2, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV> struct DFT<3, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    constexpr float c = 0.86602540378443864676f;  // sqrt(3)/2
    float2 s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    float2 t = make_float2(v[0].x - 0.5f * s.x, v[0].y - 0.5f * s.y);
    v[0] = cadd(v[0], s);
    // forward: y1 = t - i c d, y2 = t + i c d
    float2 icd = make_float2(-c * d.y, c * d.x);   // i * c * d
    if (INV) { v[1] = cadd(t, icd); v[2] = csub(t, icd); }
    else     { v[1] = csub(t, icd); v[2] = cadd(t, icd); }
  }
};

// odd prime P by symmetric pairs: y_k = v0 + sum_j cos(2 pi jk/P) a_j -+ i sum_j sin(2 pi jk/P) b_j
template <int P, bool INV> struct DFTPrime {
  template <int K, int J>
  __device__ __forceinline__ static void acc(const float2* a, const float2* b, float2& C, float2& S) {
    if constexpr (J <= (P - 1) / 2) {
      constexpr float cs = (float)ct_cos(2.0 * kPi * ((J * K) % P) / P);
      constexpr float sn = (float)ct_sin(2.0 * kPi * ((J * K) % P) / P);
      C.x += cs * a[J].x; C.y += cs * a[J].y;
      S.x += sn * b[J].x; S.y += sn * b[J].y;
      acc<K, J + 1>(a, b, C, S);
    }
  }
  template <int K>
  __device__ __forceinline__ static void out(const float2* v, const float2* a, const float2* b, float2* y) {
    if constexpr (K <= (P - 1) / 2) {
      float2 C = v[0], S = make_float2(0.f, 0.f);
      acc<K, 1>(a, b, C, S);
      // -i S = (S.y, -S.x)
      float2 miS = make_float2(S.y, -S.x);
      if (INV) { y[K] = csub(C, miS); y[P - K] = cadd(C, miS); }
      else     { y[K] = cadd(C, miS); y[P - K] = csub(C, miS); }
      out<K + 1>(v, a, b, y);
    }
  }
  __device__ __forceinline__ static void run(float2* v) {
    float2 a[(P + 1) / 2], b[(P + 1) / 2], y[P];
    float2 s0 = v[0];
#pragma unroll
    for (int j = 1; j <= (P - 1) / 2; ++j) {
      a[j] = cadd(v[j], v[P - j]);
      b[j] = csub(v[j], v[P - j]);
      s0 = cadd(s0, a[j]);
    }
    out<1>(v, a, b, y);
    y[0] = s0;
#pragma unroll
    for (int k = 0; k < P; ++k) v[k] = y[k];
  }
};
template <bool INV> struct DFT<5, INV> : DFTPrime<5, INV> {};
template <bool INV> struct DFT<7, INV> : DFTPrime<7, INV> {};

// composite R = A*B by in-register Cooley-Tukey:
// x[B*n1 + n2] --DFT_A over n1--> U[n2][k1] --*W_R^{n2*k1}--> DFT_B over n2 --> X[k1 + A*k2]
template <int A, int B, bool INV> struct DFTComposite {
  template <int N2, int K1>
  __device__ __forceinline__ static void tw(float2 (&u)[B][A]) {
    if constexpr (N2 < B) {
      if constexpr (K1 < A) {
        u[N2][K1] = twc<N2 * K1, A * B, INV>(u[N2][K1]);
        tw<N2, K1 + 1>(u);
      } else {
        tw<N2 + 1, 0>(u);
      }
    }
  }
  __device__ __forceinline__ static void run(float2* v) {
    float2 u[B][A];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) u[n2][n1] = v[B * n1 + n2];
      DFT<A, INV>::run(u[n2]);
    }
    tw<0, 0>(u);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      float2 w[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) w[n2] = u[n2][k1];
      DFT<B, INV>::run(w);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = w[k2];
    }
  }
};
// radix 4: X0 = (a+c)+(b+d), X2 = (a+c)-(b+d), X1 = (a-c) -+ i(b-d), X3 = (a-c) +- i(b-d)
// (forward upper signs); the +-i products are a swap of (b-d) and one packed
// multiply-add by (1, -1) or (-1, 1)
template <bool INV> struct DFT<4, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    const float2 s0 = cadd(v[0], v[2]), d0 = csub(v[0], v[2]);
    const float2 s1 = cadd(v[1], v[3]), d1 = csub(v[1], v[3]);
    const float2 sw = make_float2(d1.y, d1.x);
    v[0] = cadd(s0, s1);
    v[2] = csub(s0, s1);
    // forward: X1 = d0 - i d1 = (d0.x + d1.y, d0.y - d1.x)
    v[1] = INV ? cfma_lanes(sw, -1.f, 1.f, d0) : cfma_lanes(sw, 1.f, -1.f, d0);
    v[3] = INV ? cfma_lanes(sw, 1.f, -1.f, d0) : cfma_lanes(sw, -1.f, 1.f, d0);
  }
};
template <bool INV> struct DFT<6, INV> : DFTComposite<2, 3, INV> {};
template <bool INV> struct DFT<8, INV> : DFTComposite<4, 2, INV> {};
template <bool INV> struct DFT<10, INV> : DFTComposite<2, 5, INV> {};
template <bool INV> struct DFT<12, INV> : DFTComposite<4, 3, INV> {};
template <bool INV> struct DFT<16, INV> : DFTComposite<4, 4, INV> {};

// ---------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------
constexpr int kMaxStages = 8;
struct AxisPlan {
  int n;
  int nst;
  int radix[kMaxStages];
};

// ---------------------------------------------------------------------------
// I/O functors for shared-memory lines: element (line, idx) at base[line*ls + idx*es]
// ---------------------------------------------------------------------------
struct SmemLines {
  float2* base;
  int ls, es;
  __device__ __forceinline__ float2 load(int line, int idx) const {
    const float2* q = base + line * ls + idx * es;
    return PF_CHECK_SMEM(kChkSmem, q, 8) ? *q : make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ void store(int line, int idx, float2 v) const {
    float2* q = base + line * ls + idx * es;
    if (PF_CHECK_SMEM(kChkSmem, q, 8)) *q = v;
  }
};

// ---------------------------------------------------------------------------
// One Stockham stage over a batch of lines, chunked so that every item of a
// chunk is held in registers before any of it is stored (in-place safe).
// ---------------------------------------------------------------------------
template <int R, bool INV, int EMAX, class Src, class Dst>
__device__ __forceinline__ void fft_stage(int nlines, int L, int Ns, const float2* __restrict__ tw,
                                          const Src src, const Dst dst, bool alias) {
  constexpr int K = (EMAX / R) > 0 ? (EMAX / R) : 1;
  const int nb = L / R;
  const int nthreads = blockDim.x;
  int C = (nthreads * K) / nb;
  if (C > nlines) C = nlines;
  if (C < 1) C = 1;  // edges are limited on the host so that one line always fits
  const int twmul = L / (Ns * R);
  for (int l0 = 0; l0 < nlines; l0 += C) {
    const int cl = min(C, nlines - l0);
    const int items = cl * nb;
    float2 v[K][R];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int it = threadIdx.x + k * nthreads;
      if (it < items) {
        const int line = l0 + it % cl;
        const int j = it / cl;
#pragma unroll
        for (int r = 0; r < R; ++r) v[k][r] = src.load(line, j + r * nb);
        if (Ns > 1) {   // (the first stage's twiddles are all 1)
          const int jm = (j % Ns) * twmul;
#pragma unroll
          for (int r = 1; r < R; ++r) {
            float2 w = PF_CHECK(kChkTwiddle, r * jm, L) ? tw[r * jm] : make_float2(1.f, 0.f);
            if (INV) w.y = -w.y;
            v[k][r] = cmul(v[k][r], w);
          }
        }
        DFT<R, INV>::run(v[k]);
      }
    }
    if (alias) __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int it = threadIdx.x + k * nthreads;
      if (it < items) {
        const int line = l0 + it % cl;
        const int j = it / cl;
        const int base = (j / Ns) * Ns * R + (j % Ns);
#pragma unroll
        for (int r = 0; r < R; ++r) dst.store(line, base + r * Ns, v[k][r]);
      }
    }
    if (alias) __syncthreads();
  }
}

// split-bf16x3 tensor-core stage (pf_fft_mma.cuh)
template <bool INV, class Src, class Dst>
__device__ __noinline__ void fft_stage_mma(int R, int nlines, int L, int Ns, const float2* __restrict__ tw,
                                           const Src src, const Dst dst, bool alias);

// split-bf16x3 stage on the tcgen05 tensor cores (pf_fft_tc05.cuh)
template <bool INV, class Src, class Dst>
__device__ __noinline__ void fft_stage_tc05(int R, int nlines, int L, int Ns, const float2* __restrict__ tw,
                                            const Src src, const Dst dst, bool alias);

// TC: 0, the R-point DFTs in float32 codelets; 1, on the tensor cores in
// split-bf16x3 with mma.sync; 2, the same products with tcgen05.mma (both
// precision-study variants)
template <bool INV, int EMAX, int TC, class Src, class Dst>
__device__ __noinline__ void fft_stage_rt(int R, int nlines, int L, int Ns, const float2* __restrict__ tw,
                                          const Src src, const Dst dst, bool alias) {
  if constexpr (TC == 2) {
    if (R > 1) {
      fft_stage_tc05<INV>(R, nlines, L, Ns, tw, src, dst, alias);
      return;
    }
  } else if constexpr (TC == 1) {
    if (R > 1) {
      fft_stage_mma<INV>(R, nlines, L, Ns, tw, src, dst, alias);
      return;
    }
  }
  switch (R) {
    case 16: fft_stage<16, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
    case 12: fft_stage<12, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
    case 10: fft_stage<10, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
    case 8: fft_stage<8, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
    case 7: fft_stage<7, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
    case 6: fft_stage<6, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
    case 5: fft_stage<5, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
    case 4: fft_stage<4, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
    case 3: fft_stage<3, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
    case 2: fft_stage<2, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
    default: fft_stage<1, INV, EMAX>(nlines, L, Ns, tw, src, dst, alias); break;
  }
}

// Full transform of `nlines` lines of length pl.n: the first stage reads from
// `src`, the last writes to `dst`, intermediate stages work in `mid` (shared
// memory).  `src_alias`/`dst_alias`: whether src/dst share storage with `mid`.
template <bool INV, int EMAX, int TC = 0, class Src, class Mid, class Dst>
__device__ __forceinline__ void fft_lines(const AxisPlan& pl, int nlines, const float2* __restrict__ tw,
                                          const Src src, const Mid mid, const Dst dst,
                                          bool src_alias, bool dst_alias) {
  int Ns = 1;
  const int L = pl.n;
  if (pl.nst == 1) {
    fft_stage_rt<INV, EMAX, TC>(pl.radix[0], nlines, L, 1, tw, src, dst, src_alias || dst_alias);
    return;
  }
  for (int s = 0; s < pl.nst; ++s) {
    const int R = pl.radix[s];
    if (s == 0) fft_stage_rt<INV, EMAX, TC>(R, nlines, L, Ns, tw, src, mid, src_alias);
    else if (s == pl.nst - 1) fft_stage_rt<INV, EMAX, TC>(R, nlines, L, Ns, tw, mid, dst, dst_alias);
    else fft_stage_rt<INV, EMAX, TC>(R, nlines, L, Ns, tw, mid, mid, true);
    Ns *= R;
    __syncthreads();
  }
}

}  // namespace pf
