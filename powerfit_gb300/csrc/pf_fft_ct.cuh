// Compile-time-planned shared-memory FFT stages (sm_103a fast path).
//
// Same Stockham formulation as pf_fft.cuh, but the transform length, the
// radix sequence, the thread count and the chunk geometry are template
// constants: every index computation reduces to shifts and multiplies, the
// per-thread value arrays stay in registers, and the stages inline into the
// kernels.  Lines are mapped to threads line-fastest (consecutive threads take
// consecutive lines), so with an odd row stride every access is free of
// shared-memory bank conflicts whatever the index pattern of the stage.
#pragma once
#include <type_traits>
#include "pf_fft.cuh"

namespace pf {

// Threads that run a transform together, and their barrier.  BlockTeam: the
// whole block (__syncthreads).  GroupTeam<NTT>: the block split into teams of
// NTT consecutive threads (whole warps), team t synchronising on named barrier
// 1 + t alone, so that teams working on disjoint lines run their stages out of
// step with each other (one team's loads beside another's arithmetic).
struct BlockTeam {
  static __device__ __forceinline__ int tid() { return threadIdx.x; }
  static __device__ __forceinline__ void sync() { __syncthreads(); }
};
template <int NTT>
struct GroupTeam {
  static_assert(NTT % 32 == 0, "a team is whole warps");
  static __device__ __forceinline__ int tid() { return threadIdx.x % NTT; }
  static __device__ __forceinline__ int team() { return threadIdx.x / NTT; }
  static __device__ __forceinline__ void sync() {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + (int)(threadIdx.x / NTT)), "n"(NTT) : "memory");
  }
};

struct CtPlan {
  int n;
  int nst;
  int r[kMaxStages];
};

// fewest stages, then the largest smallest radix (same rule as the host planner)
constexpr int kCtRadices[10] = {16, 12, 10, 8, 7, 6, 5, 4, 3, 2};

struct CtSearch {
  int best[kMaxStages];
  int best_n;
  int best_min;
  int cur[kMaxStages];
  int cur_n;
};

constexpr void ct_rec(CtSearch& s, int rem, int maxr) {
  if (rem == 1) {
    if (s.cur_n == 0) return;
    int mn = 1 << 30;
    for (int i = 0; i < s.cur_n; ++i) mn = s.cur[i] < mn ? s.cur[i] : mn;
    if (s.best_n == 0 || s.cur_n < s.best_n || (s.cur_n == s.best_n && mn > s.best_min)) {
      for (int i = 0; i < s.cur_n; ++i) s.best[i] = s.cur[i];
      s.best_n = s.cur_n;
      s.best_min = mn;
    }
    return;
  }
  if (s.best_n != 0 && s.cur_n + 1 > s.best_n) return;
  if (s.cur_n >= kMaxStages) return;
  for (int k = 0; k < 10; ++k) {
    const int r = kCtRadices[k];
    if (r > maxr || rem % r) continue;
    s.cur[s.cur_n++] = r;
    ct_rec(s, rem / r, r);
    s.cur_n--;
  }
}

constexpr CtPlan ct_plan(int n) {
  CtPlan p{};
  p.n = n;
  if (n == 1) {
    p.nst = 1;
    p.r[0] = 1;
    return p;
  }
  CtSearch s{};
  ct_rec(s, n, 16);
  p.nst = s.best_n;
  for (int i = 0; i < s.best_n; ++i) p.r[i] = s.best[i];
  return p;
}

constexpr int ct_stage_ns(int n, int stage) {
  CtPlan p = ct_plan(n);
  int ns = 1;
  for (int i = 0; i < stage; ++i) ns *= p.r[i];
  return ns;
}

constexpr int ct_floor_pow2(int v) {
  int p = 1;
  while (p * 2 <= v) p *= 2;
  return p;
}

constexpr int ct_log2(int v) {
  int l = 0;
  while ((1 << (l + 1)) <= v) ++l;
  return l;
}

// One radix-R stage over `nlines` lines of length L.  Lines are processed in
// chunks of C (a power of two) lines, mapped line-fastest (consecutive threads
// take consecutive lines); every item (line, butterfly) of a chunk is loaded
// into registers before any is stored, so src and dst may alias.  A last,
// partial chunk of at most C/2 lines is mapped as C/2 lines: its items then
// fill whole warps and the other warps wait at the barrier instead of issuing
// with half their lanes off (48 lines: 32 + 16).
template <int R, bool INV, int L, int NS, int NT, int EMAX, class TM = BlockTeam, class Src, class Dst>
__device__ __forceinline__ void ct_stage(int nlines, const float2* __restrict__ tw, const Src& src, const Dst& dst,
                                         bool alias) {
  constexpr int NB = L / R;
  constexpr int KMAX = (EMAX / R) > 0 ? (EMAX / R) : 1;
  constexpr int C0 = (NT * KMAX) / NB;
  constexpr int C = ct_floor_pow2(C0 > 0 ? C0 : 1);
  constexpr int LOG2C = ct_log2(C);
  constexpr int K = (C * NB + NT - 1) / NT;          // items per thread per chunk
  constexpr int TWMUL = L / (NS * R);
  // The last stage (Ns * R == L) stores every item exactly where it loaded it
  // (y[j + r Ns] with Ns == L/R), so no item can overwrite another's input:
  // it needs no barrier between its loads and its stores.
  constexpr bool kSelfInPlace = (NS * R == L);
  if (kSelfInPlace) alias = false;
  for (int l0 = 0; l0 < nlines; l0 += C) {
    // lines this chunk maps: C, or C/2 for a short last chunk
    const int sh = (C >= 2 && nlines - l0 <= C / 2) ? LOG2C - 1 : LOG2C;
    const int cm = (1 << sh) - 1;
    float2 v[K][R];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int it = TM::tid() + k * NT;
      const int line = l0 + (it & cm);
      const int j = it >> sh;
      if (j < NB && line < nlines) {
#pragma unroll
        for (int r = 0; r < R; ++r) v[k][r] = src.load(line, j + r * NB);
        if constexpr (NS > 1) {
          const int jm = (j % NS) * TWMUL;
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
    if (alias) TM::sync();
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int it = TM::tid() + k * NT;
      const int line = l0 + (it & cm);
      const int j = it >> sh;
      if (j < NB && line < nlines) {
        const int base = (j / NS) * NS * R + (j % NS);
#pragma unroll
        for (int r = 0; r < R; ++r) dst.store(line, base + r * NS, v[k][r]);
      }
    }
    if (alias) TM::sync();
  }
}

template <int L, bool INV, int NT, int EMAX, int S, class TM, class Src, class Mid, class Dst>
__device__ __forceinline__ void ct_lines_from(int nlines, const float2* __restrict__ tw, const Src& src,
                                              const Mid& mid, const Dst& dst, bool src_alias, bool dst_alias) {
  constexpr CtPlan P = ct_plan(L);
  if constexpr (S < P.nst) {
    constexpr int R = P.r[S];
    constexpr int NS = ct_stage_ns(L, S);
    if constexpr (P.nst == 1) {
      ct_stage<R, INV, L, NS, NT, EMAX, TM>(nlines, tw, src, dst, src_alias || dst_alias);
    } else if constexpr (S == 0) {
      ct_stage<R, INV, L, NS, NT, EMAX, TM>(nlines, tw, src, mid, src_alias);
      TM::sync();
    } else if constexpr (S == P.nst - 1) {
      ct_stage<R, INV, L, NS, NT, EMAX, TM>(nlines, tw, mid, dst, dst_alias);
    } else {
      ct_stage<R, INV, L, NS, NT, EMAX, TM>(nlines, tw, mid, mid, true);
      TM::sync();
    }
    ct_lines_from<L, INV, NT, EMAX, S + 1, TM>(nlines, tw, src, mid, dst, src_alias, dst_alias);
  }
}

// Full length-L transform of `nlines` lines: first stage reads `src`, last
// writes `dst`, the others work in `mid` (shared memory).  Ends with a barrier.
template <int L, bool INV, int NT, int EMAX, class TM = BlockTeam, class Src, class Mid, class Dst>
__device__ __forceinline__ void ct_lines(int nlines, const float2* __restrict__ tw, const Src& src, const Mid& mid,
                                         const Dst& dst, bool src_alias, bool dst_alias) {
  ct_lines_from<L, INV, NT, EMAX, 0, TM>(nlines, tw, src, mid, dst, src_alias, dst_alias);
  TM::sync();
}


// Forward stages 0 .. nst-2 in place (all but the last); stage 0 reads `src`
// (which aliases `mid` when `src_alias`).
template <int L, int NT, int EMAX, int S, class TM, class Src, class Mid>
__device__ __forceinline__ void ct_fwd_head(int nlines, const float2* __restrict__ tw, const Src& src,
                                            const Mid& mid, bool src_alias) {
  constexpr CtPlan P = ct_plan(L);
  if constexpr (S < P.nst - 1) {
    constexpr int R = P.r[S];
    constexpr int NS = ct_stage_ns(L, S);
    if constexpr (S == 0) ct_stage<R, false, L, NS, NT, EMAX, TM>(nlines, tw, src, mid, src_alias);
    else ct_stage<R, false, L, NS, NT, EMAX, TM>(nlines, tw, mid, mid, true);
    TM::sync();
    ct_fwd_head<L, NT, EMAX, S + 1, TM>(nlines, tw, src, mid, src_alias);
  }
}

// Stages 0 .. nst-2 of a length-L transform, in place in `mid`, each followed
// by a barrier.
template <int L, bool INV, int NT, int EMAX, int S, class TM = BlockTeam, class Mid>
__device__ __forceinline__ void ct_head_inplace(int nlines, const float2* __restrict__ tw, const Mid& mid) {
  constexpr CtPlan P = ct_plan(L);
  if constexpr (S < P.nst - 1) {
    constexpr int R = P.r[S];
    constexpr int NS = ct_stage_ns(L, S);
    ct_stage<R, INV, L, NS, NT, EMAX, TM>(nlines, tw, mid, mid, true);
    TM::sync();
    ct_head_inplace<L, INV, NT, EMAX, S + 1, TM>(nlines, tw, mid);
  }
}

// Twiddles of the last stage as an [r][j] table: tl[r * NB + j] = tw[r * j],
// NB = L / R_last (the last stage has Ns = NB, so butterfly j of it multiplies
// input r by tw[r * j]).
template <int L, int NT>
__device__ __forceinline__ void ct_last_twiddles(const float2* __restrict__ tw, float2* tl) {
  constexpr CtPlan P = ct_plan(L);
  constexpr int NB = L / P.r[P.nst - 1];
  for (int i = threadIdx.x; i < L; i += NT) {
    const int r = i / NB, j = i - r * NB;
    if (PF_CHECK(kChkTwiddle, r * j, L) && PF_CHECK_SMEM(kChkSmem, tl + i, 8)) tl[i] = tw[r * j];
  }
}

// Last stage of a length-L transform with the items mapped butterfly-fastest
// (consecutive threads take consecutive butterflies j of one line), reading
// `mid` and writing `out`.  Its stores y[j + r Ns] from consecutive threads
// cover consecutive elements of a line, so `out` may be global memory, written
// in whole segments straight from registers.  `tl` is the [r][j] table above.
template <int L, bool INV, int NT, class TM = BlockTeam, class Mid, class Out>
__device__ __forceinline__ void ct_last_stage_out(int nlines, const float2* __restrict__ tl, const Mid& mid,
                                                  const Out& out) {
  constexpr CtPlan P = ct_plan(L);
  constexpr int R = P.r[P.nst - 1];
  constexpr int NB = L / R;
  const int total = nlines * NB;
  for (int it = TM::tid(); it < total; it += NT) {
    const int line = it / NB, j = it - line * NB;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = mid.load(line, j + r * NB);
    if constexpr (P.nst > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = PF_CHECK(kChkTwiddle, r * NB + j, L) ? tl[r * NB + j] : make_float2(1.f, 0.f);
        if (INV) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    DFT<R, INV>::run(v);
#pragma unroll
    for (int r = 0; r < R; ++r) out.store(line, j + r * NB, v[r]);
  }
}

// Reversed radix plan (any radix order is a valid Stockham plan): used for the
// inverse transform that follows a forward one, so that the inverse's first
// stage consumes exactly the values the forward's last stage produced.
constexpr CtPlan ct_plan_rev(int n) {
  CtPlan p = ct_plan(n);
  CtPlan q = p;
  for (int i = 0; i < p.nst; ++i) q.r[i] = p.r[p.nst - 1 - i];
  return q;
}

constexpr int ct_stage_ns_rev(int n, int stage) {
  CtPlan q = ct_plan_rev(n);
  int ns = 1;
  for (int i = 0; i < stage; ++i) ns *= q.r[i];
  return ns;
}

// Stages S .. nst-1 of the reversed plan, in place in `mid`; the last one
// stores to `dst` instead when `kToDst` (a different memory: no barrier
// between its loads and stores, none after it).
template <int L, bool INV, int NT, int EMAX, int S, bool kToDst = false, class TM = BlockTeam, class Mid,
          class Dst = Mid>
__device__ __forceinline__ void ct_rev_from(int nlines, const float2* __restrict__ tw, const Mid& mid,
                                            const Dst& dst = Dst{}) {
  constexpr CtPlan Q = ct_plan_rev(L);
  if constexpr (S < Q.nst) {
    constexpr int R = Q.r[S];
    constexpr int NS = ct_stage_ns_rev(L, S);
    if constexpr (kToDst && S == Q.nst - 1) {
      ct_stage<R, INV, L, NS, NT, EMAX, TM>(nlines, tw, mid, dst, false);
    } else {
      ct_stage<R, INV, L, NS, NT, EMAX, TM>(nlines, tw, mid, mid, true);
      TM::sync();
      ct_rev_from<L, INV, NT, EMAX, S + 1, kToDst, TM>(nlines, tw, mid, dst);
    }
  }
}

// Forward transform, pointwise product, inverse transform of `nlines` lines
// held in shared memory (`mid`).  The forward's last stage, the product
// ``mul(line, k, v)`` and the inverse's first stage (reversed plan) run on the
// same registers: radix R_last with Ns = L/R_last stores y[j + r L/R], which
// is exactly what a first stage (Ns = 1) of radix R_last loads.
//
// The forward's first stage reads `src` (by default `mid` itself); `src_alias`
// says whether it shares memory with `mid`.
//
// With a `Dst` other than `void`, the inverse's last stage stores to `dst`
// (the plan must have at least two stages) and no barrier follows it.
template <int L, int NT, int EMAX, class TM = BlockTeam, class Mid, class Mul, class Src = Mid, class Dst = void>
__device__ __forceinline__ void ct_fwd_mul_inv(int nlines, const float2* __restrict__ tw, const Mid& mid,
                                               const Mul& mul, const Src& src, bool src_alias,
                                               const Dst* dstp = nullptr) {
  constexpr CtPlan P = ct_plan(L);
  constexpr int RL = P.r[P.nst - 1];
  constexpr int NB = L / RL;
  // forward stages 0 .. nst-2
  ct_fwd_head<L, NT, EMAX, 0, TM>(nlines, tw, src, mid, src_alias);
  // fused stage
  constexpr int KMAX = (EMAX / RL) > 0 ? (EMAX / RL) : 1;
  constexpr int C0 = (NT * KMAX) / NB;
  constexpr int C = ct_floor_pow2(C0 > 0 ? C0 : 1);
  constexpr int K = (C * NB + NT - 1) / NT;
  for (int l0 = 0; l0 < nlines; l0 += C) {
    float2 v[K][RL];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int it = TM::tid() + k * NT;
      const int line = l0 + (it & (C - 1));
      const int j = it / C;
      if (j < NB && line < nlines) {
        float2 m[RL];
#pragma unroll
        for (int r = 0; r < RL; ++r) m[r] = mul.fetch(line, j + r * NB);   // issue the operand loads early
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          if constexpr (P.nst == 1) v[k][r] = src.load(line, j + r * NB);   // the only stage is the first
          else v[k][r] = mid.load(line, j + r * NB);
        }
        if constexpr (NB > 1) {           // forward last stage twiddles (Ns = NB)
          const int jm = j;               // (j % NB) * (L / (NB * RL)) with L / (NB * RL) == 1
#pragma unroll
          for (int r = 1; r < RL; ++r)
            v[k][r] = cmul(v[k][r], PF_CHECK(kChkTwiddle, r * jm, L) ? tw[r * jm] : make_float2(1.f, 0.f));
        }
        DFT<RL, false>::run(v[k]);
#pragma unroll
        for (int r = 0; r < RL; ++r) v[k][r] = cmulc(v[k][r], m[r]);
        DFT<RL, true>::run(v[k]);         // inverse first stage (Ns = 1): no twiddles
      }
    }
    TM::sync();
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int it = TM::tid() + k * NT;
      const int line = l0 + (it & (C - 1));
      const int j = it / C;
      if (j < NB && line < nlines) {
#pragma unroll
        for (int r = 0; r < RL; ++r) mid.store(line, j * RL + r, v[k][r]);
      }
    }
    TM::sync();
  }
  // inverse stages 1 .. nst-1 of the reversed plan
  if constexpr (std::is_void<Dst>::value) {
    ct_rev_from<L, true, NT, EMAX, 1, false, TM>(nlines, tw, mid);
  } else {
    static_assert(P.nst >= 2, "the last inverse stage must not be the fused one");
    ct_rev_from<L, true, NT, EMAX, 1, true, TM>(nlines, tw, mid, *dstp);
  }
}

}  // namespace pf
