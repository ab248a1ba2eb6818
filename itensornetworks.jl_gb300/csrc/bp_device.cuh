// Shared-memory fiber primitives of the SIMT belief-propagation kernels
// (ABSORB a message into one leg of a vertex tensor, CLOSE a tensor against the
// bra on one leg), team synchronisation, warp reductions and the per-team
// shared-memory carve-up.  Included by bp_kernels.cu and adjoint.cu.
#pragma once

#include <type_traits>

#include "gbtn_internal.h"

namespace gbtn {

// ---------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------

template <int TEAM>
__device__ __forceinline__ void tsync() {
  if constexpr (TEAM == 32)
    __syncwarp();
  else
    __syncthreads();
}

// Arithmetic of the complex FP64 element (zdouble, gbtn_internal.h) that the
// fiber primitives need.  The bra of the quadratic form is conj(tensor) (dag
// in the reference), which is the identity for real element types.
__device__ __forceinline__ zdouble operator+(zdouble a, zdouble b) { return zdouble(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ zdouble& operator+=(zdouble& a, zdouble b) {
  a.re += b.re;
  a.im += b.im;
  return a;
}
__device__ __forceinline__ zfloat operator+(zfloat a, zfloat b) { return zfloat(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ zfloat& operator+=(zfloat& a, zfloat b) {
  a.re += b.re;
  a.im += b.im;
  return a;
}
// Double-FP32 element ("double-float"): the unevaluated sum hi + lo of two
// floats, about 48 significant bits, carried on the FP32 pipe.  GB300's FP32
// pipe issues 64 times the FP64 rate, so the refinement sweeps that need more
// than FP32 accuracy run in this arithmetic (tensors and messages stay FP64 in
// HBM and are split on load; norms and message diffs are formed in FP64).
// The operations are the error-free transformations of Knuth (TwoSum) and
// Dekker (1971) / Ogita, Rump & Oishi (2005) (the product error from one FMA):
//   mac(a, b, c): p = a.hi b.hi exactly split into p + e by an FMA, the cross
//   terms a.hi b.lo + a.lo b.hi folded into e, then TwoSum(c.hi, p) with the
//   low parts summed into the error word.  mac leaves (hi, lo) unnormalised
//   (|lo| may exceed half an ulp of hi); settle() renormalises with a
//   FastTwoSum before a value is stored or reused as an operand.
struct __align__(8) df32 {
  float hi, lo;
  df32() = default;
  __host__ __device__ constexpr df32(float h, float l = 0.f) : hi(h), lo(l) {}
};

__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ df32 settle(df32 a) {
  const float s = __fadd_rn(a.hi, a.lo);
  return df32(s, __fsub_rn(a.lo, __fsub_rn(s, a.hi)));
}
__device__ __forceinline__ df32 operator+(df32 a, df32 b) {
  float s, e;
  df_two_sum(a.hi, b.hi, s, e);
  return settle(df32(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo))));
}
__device__ __forceinline__ df32& operator+=(df32& a, df32 b) {
  a = a + b;
  return a;
}
__device__ __forceinline__ df32 mac(df32 a, df32 b, df32 c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  float s, t;
  df_two_sum(c.hi, p, s, t);
  return df32(s, __fadd_rn(__fadd_rn(t, e), c.lo));
}
// Two independent df32 values per register pair, for the packed FP32x2
// instructions: the same operations as mac() and settle(), each component
// rounded exactly as there.  A difference x - y is the FMA y * (-1) + x (one
// rounding, as __fsub_rn); the product error is carried negated, en = -e, so
// that no operand needs a negation of its own.
struct df32x2 {
  float2 hi, lo;
};
__device__ __forceinline__ float2 sub2(float2 x, float2 y) { return __ffma2_rn(y, make_float2(-1.f, -1.f), x); }
// a * (bh + bl) + c for a pair a, c and one value b given with its negation (nbh, nbl)
__device__ __forceinline__ df32x2 mac2(const df32x2& a, float2 bh, float2 nbh, float2 nbl, const df32x2& c) {
  const float2 p = __fmul2_rn(a.hi, bh);
  float2 en = __ffma2_rn(a.hi, nbh, p);
  en = __ffma2_rn(a.hi, nbl, en);
  en = __ffma2_rn(a.lo, nbh, en);
  const float2 s = __fadd2_rn(c.hi, p);
  const float2 bb = sub2(s, c.hi);
  const float2 t = __fadd2_rn(sub2(c.hi, sub2(s, bb)), sub2(p, bb));
  return df32x2{s, __fadd2_rn(sub2(t, en), c.lo)};
}
__device__ __forceinline__ df32x2 settle2(const df32x2& a) {
  const float2 s = __fadd2_rn(a.hi, a.lo);
  return df32x2{s, sub2(a.lo, sub2(s, a.hi))};
}

__device__ __forceinline__ df32 conj_of(df32 x) { return x; }
__device__ __forceinline__ df32 shfl_xor(df32 v, int o) {
  return df32(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}
__device__ __forceinline__ df32 df_from_double(double x) {
  const float h = __double2float_rn(x);
  return df32(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ double df_to_double(df32 a) { return (double)a.hi + (double)a.lo; }

// Storage element -> arithmetic element (identity unless the arithmetic is df32).
template <typename T, typename S>
__device__ __forceinline__ T to_elem(S x) {
  if constexpr (std::is_same<T, df32>::value)
    return df_from_double(x);
  else
    return x;
}
template <typename T>
__device__ __forceinline__ T settle(T x) {
  return x;
}

// multiply-accumulate a * b + c
__device__ __forceinline__ float mac(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double mac(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ zdouble mac(zdouble a, zdouble b, zdouble c) {
  return zdouble(fma(a.re, b.re, fma(-a.im, b.im, c.re)), fma(a.re, b.im, fma(a.im, b.re, c.im)));
}
__device__ __forceinline__ zfloat mac(zfloat a, zfloat b, zfloat c) {
  return zfloat(fmaf(a.re, b.re, fmaf(-a.im, b.im, c.re)), fmaf(a.re, b.im, fmaf(a.im, b.re, c.im)));
}
__device__ __forceinline__ float conj_of(float x) { return x; }
__device__ __forceinline__ double conj_of(double x) { return x; }
__device__ __forceinline__ zdouble conj_of(zdouble x) { return zdouble(x.re, -x.im); }
__device__ __forceinline__ zfloat conj_of(zfloat x) { return zfloat(x.re, -x.im); }
__device__ __forceinline__ float shfl_xor(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ zdouble shfl_xor(zdouble v, int o) {
  return zdouble(__shfl_xor_sync(0xffffffffu, v.re, o), __shfl_xor_sync(0xffffffffu, v.im, o));
}
__device__ __forceinline__ zfloat shfl_xor(zfloat v, int o) {
  return zfloat(__shfl_xor_sync(0xffffffffu, v.re, o), __shfl_xor_sync(0xffffffffu, v.im, o));
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Reduce-scatter of P2 values over a warp: afterwards lane L holds the
// warp-wide sums of entries [L*P2/32, (L+1)*P2/32) in v[0 .. P2/32).
template <typename T, int P2>
__device__ __forceinline__ void warp_reduce_scatter(T (&v)[P2], int lane) {
  // step s (lane bit 4 - s): while more than one value is left, each lane keeps
  // the half its lane bit selects and adds its partner's copy of that half;
  // with one value left, a plain butterfly sum over the remaining lane bits
#pragma unroll
  for (int step = 0; step < 5; ++step) {
    const int h = P2 >> (step + 1);
    const int mask = 16 >> step;
    if (h == 0) {
      v[0] = v[0] + shfl_xor(v[0], mask);
      continue;
    }
    const bool upper = (lane & mask) != 0;
#pragma unroll
    for (int i = 0; i < P2 / 2; ++i) {
      if (i < h) {
        T send = upper ? v[i] : v[i + h];
        T keep = upper ? v[i + h] : v[i];
        v[i] = keep + shfl_xor(send, mask);
      }
    }
  }
}

// Shared-memory position of tensor element i.  With PAD one unused element
// follows every 32: the fibers of the innermost legs (strides 2 and 16 at
// d = 2, chi = 8) then spread a warp over many banks instead of 2-4 (an
// 8-way conflict on leg 0 without it).  padded_len(n) elements hold a padded
// tensor of n elements.
template <bool PAD>
__device__ __forceinline__ int spos(int i) {
  if constexpr (PAD)
    return i + (i >> 5);
  else
    return i;
}
__host__ __device__ inline int padded_len(int n) { return n + (n >> 5) + 1; }

// FP32 fibers use the packed FP32x2 FMA (two outputs b, b + 1 per
// instruction, each component rounded as one fmaf, in the same order).
template <int CHI, bool PAD>
__device__ __forceinline__ void absorb_fibers_f32x2(const float* __restrict__ in, float* __restrict__ out, int n,
                                                    int st, const float* __restrict__ M, int tid, int nth) {
  constexpr int H = (CHI + 1) / 2;
  float2 m[H][CHI];
#pragma unroll
  for (int h = 0; h < H; ++h)
#pragma unroll
    for (int a = 0; a < CHI; ++a)
      m[h][a] = make_float2(M[2 * h + CHI * a], 2 * h + 1 < CHI ? M[2 * h + 1 + CHI * a] : 0.f);
  const int nfib = n / CHI;
  for (int f = tid; f < nfib; f += nth) {
    const int lo = f % st;
    const int base = lo + (f - lo) * CHI;
    float x[CHI];
#pragma unroll
    for (int a = 0; a < CHI; ++a) x[a] = in[spos<PAD>(base + a * st)];
#pragma unroll
    for (int h = 0; h < H; ++h) {
      float2 y = make_float2(0.f, 0.f);
#pragma unroll
      for (int a = 0; a < CHI; ++a) y = __ffma2_rn(m[h][a], make_float2(x[a], x[a]), y);
      out[spos<PAD>(base + 2 * h * st)] = y.x;
      if (2 * h + 1 < CHI) out[spos<PAD>(base + (2 * h + 1) * st)] = y.y;
    }
  }
}

// df32 fibers: outputs b, b + 1 as one df32x2 (mac2, settle2).  Taken by
// one-warp teams (PACK); a 256-thread team, one block per SM, keeps the
// scalar loop, whose eight independent chains per fiber hide the FP32
// latency better than four packed ones (measured on both kinds of vertex).
template <int CHI, bool PAD>
__device__ __forceinline__ void absorb_fibers_df32x2(const df32* __restrict__ in, df32* __restrict__ out, int n,
                                                     int st, const df32* __restrict__ M, int tid, int nth) {
  constexpr int H = (CHI + 1) / 2;
  df32x2 m[H][CHI];
#pragma unroll
  for (int h = 0; h < H; ++h)
#pragma unroll
    for (int a = 0; a < CHI; ++a) {
      const df32 u = M[2 * h + CHI * a];
      const df32 w = 2 * h + 1 < CHI ? M[2 * h + 1 + CHI * a] : df32(0.f);
      m[h][a] = df32x2{make_float2(u.hi, w.hi), make_float2(u.lo, w.lo)};
    }
  const int nfib = n / CHI;
  for (int f = tid; f < nfib; f += nth) {
    const int lo = f % st;
    const int base = lo + (f - lo) * CHI;
    df32 x[CHI];
#pragma unroll
    for (int a = 0; a < CHI; ++a) x[a] = in[spos<PAD>(base + a * st)];
#pragma unroll
    for (int h = 0; h < H; ++h) {
      df32x2 y{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
      for (int a = 0; a < CHI; ++a)
        y = mac2(m[h][a], make_float2(x[a].hi, x[a].hi), make_float2(-x[a].hi, -x[a].hi),
                 make_float2(-x[a].lo, -x[a].lo), y);
      y = settle2(y);
      out[spos<PAD>(base + 2 * h * st)] = df32(y.hi.x, y.lo.x);
      if (2 * h + 1 < CHI) out[spos<PAD>(base + (2 * h + 1) * st)] = df32(y.hi.y, y.lo.y);
    }
  }
}

template <typename T, int CHI, bool PAD = false, bool PACK = false>
__device__ __forceinline__ void absorb_fibers(const T* __restrict__ in, T* __restrict__ out, int n, int st,
                                              const T* __restrict__ M, int tid, int nth) {
  if constexpr (std::is_same<T, float>::value && CHI > 1) {
    absorb_fibers_f32x2<CHI, PAD>(in, out, n, st, M, tid, nth);
  } else if constexpr (std::is_same<T, df32>::value && CHI > 1 && PACK) {
    absorb_fibers_df32x2<CHI, PAD>(in, out, n, st, M, tid, nth);
  } else {
    T m[CHI][CHI];
#pragma unroll
    for (int b = 0; b < CHI; ++b)
#pragma unroll
      for (int a = 0; a < CHI; ++a) m[b][a] = M[b + CHI * a];
    const int nfib = n / CHI;
    for (int f = tid; f < nfib; f += nth) {
      const int lo = f % st;
      const int base = lo + (f - lo) * CHI;
      T x[CHI];
#pragma unroll
      for (int a = 0; a < CHI; ++a) x[a] = in[spos<PAD>(base + a * st)];
#pragma unroll
      for (int b = 0; b < CHI; ++b) {
        T y = T(0);
#pragma unroll
        for (int a = 0; a < CHI; ++a) y = mac(m[b][a], x[a], y);
        out[spos<PAD>(base + b * st)] = settle(y);
      }
    }
  }
}

template <typename T, bool PAD = false, bool PACK = false>
__device__ __forceinline__ void absorb_any(int chi, const T* in, T* out, int n, int st, const T* M, int tid,
                                           int nth) {
  switch (chi) {
    case 1: absorb_fibers<T, 1, PAD, PACK>(in, out, n, st, M, tid, nth); break;
    case 2: absorb_fibers<T, 2, PAD, PACK>(in, out, n, st, M, tid, nth); break;
    case 3: absorb_fibers<T, 3, PAD, PACK>(in, out, n, st, M, tid, nth); break;
    case 4: absorb_fibers<T, 4, PAD, PACK>(in, out, n, st, M, tid, nth); break;
    case 5: absorb_fibers<T, 5, PAD, PACK>(in, out, n, st, M, tid, nth); break;
    case 6: absorb_fibers<T, 6, PAD, PACK>(in, out, n, st, M, tid, nth); break;
    case 7: absorb_fibers<T, 7, PAD, PACK>(in, out, n, st, M, tid, nth); break;
    case 8: absorb_fibers<T, 8, PAD, PACK>(in, out, n, st, M, tid, nth); break;
    default: break;
  }
}

constexpr int kRedStride = 64;  // per-warp slot of the close reduction (CHI <= 8)

// CLOSE over fibers ff = fib_add + fib_mul*f of leg (st, CHI); result
// res[b + CHI*a] = sum bra[base+shift+b*st] * t[base+a*st] (team-wide sum).
template <typename T, int CHI, int TEAM, bool PAD = false, bool PACK = false>
__device__ __forceinline__ void close_fibers(const T* __restrict__ t, const T* __restrict__ bra, int n, int st,
                                             int fib_mul, int fib_add, int bra_shift, T* red, T* res,
                                             int tid) {
  constexpr int P = CHI * CHI;
  // accumulators padded to a power of two (the reduce-scatter's shape)
  constexpr int P2 = P <= 1 ? 1 : P <= 4 ? 4 : P <= 16 ? 16 : P <= 32 ? 32 : 64;
  T acc[P2];
#pragma unroll
  for (int i = 0; i < P2; ++i) acc[i] = T(0);
  const int nfib = n / (CHI * fib_mul);
  // fiber ff of leg (st, CHI) -> its first element
  auto fiber_base = [&](int f) {
    const int ff = fib_add + fib_mul * f;
    const int lo = ff % st;
    return lo + (ff - lo) * CHI;
  };
  if constexpr (std::is_same<T, float>::value && CHI % 2 == 0) {
    // packed FP32x2 accumulators: pair (h, a) holds entries 2h + CHI a and 2h + 1 + CHI a,
    // each updated by the same fmaf sequence as the scalar loop
    constexpr int H = CHI / 2;
    float2 acc2[H][CHI];
#pragma unroll
    for (int h = 0; h < H; ++h)
#pragma unroll
      for (int a = 0; a < CHI; ++a) acc2[h][a] = make_float2(0.f, 0.f);
    for (int f = tid; f < nfib; f += TEAM) {
      const int base = fiber_base(f);
      float x[CHI];
      float2 y2[H];
#pragma unroll
      for (int a = 0; a < CHI; ++a) x[a] = t[spos<PAD>(base + a * st)];
#pragma unroll
      for (int h = 0; h < H; ++h)
        y2[h] = make_float2(bra[spos<PAD>(base + bra_shift + 2 * h * st)],
                            bra[spos<PAD>(base + bra_shift + (2 * h + 1) * st)]);
#pragma unroll
      for (int a = 0; a < CHI; ++a) {
        const float2 xa = make_float2(x[a], x[a]);
#pragma unroll
        for (int h = 0; h < H; ++h) acc2[h][a] = __ffma2_rn(y2[h], xa, acc2[h][a]);
      }
    }
#pragma unroll
    for (int h = 0; h < H; ++h)
#pragma unroll
      for (int a = 0; a < CHI; ++a) {
        acc[2 * h + CHI * a] = acc2[h][a].x;
        acc[2 * h + 1 + CHI * a] = acc2[h][a].y;
      }
  } else if constexpr (std::is_same<T, df32>::value && CHI % 2 == 0 && PACK) {
    constexpr int H = CHI / 2;
    df32x2 acc2[H][CHI];
#pragma unroll
    for (int h = 0; h < H; ++h)
#pragma unroll
      for (int a = 0; a < CHI; ++a) acc2[h][a] = df32x2{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    for (int f = tid; f < nfib; f += TEAM) {
      const int base = fiber_base(f);
      df32 x[CHI];
      df32x2 y2[H];
#pragma unroll
      for (int a = 0; a < CHI; ++a) x[a] = t[spos<PAD>(base + a * st)];
#pragma unroll
      for (int h = 0; h < H; ++h) {
        const df32 u = bra[spos<PAD>(base + bra_shift + 2 * h * st)];
        const df32 w = bra[spos<PAD>(base + bra_shift + (2 * h + 1) * st)];
        y2[h] = df32x2{make_float2(u.hi, w.hi), make_float2(u.lo, w.lo)};
      }
#pragma unroll
      for (int a = 0; a < CHI; ++a) {
        const float2 bh = make_float2(x[a].hi, x[a].hi);
        const float2 nbh = make_float2(-x[a].hi, -x[a].hi), nbl = make_float2(-x[a].lo, -x[a].lo);
#pragma unroll
        for (int h = 0; h < H; ++h) acc2[h][a] = mac2(y2[h], bh, nbh, nbl, acc2[h][a]);
      }
    }
#pragma unroll
    for (int h = 0; h < H; ++h)
#pragma unroll
      for (int a = 0; a < CHI; ++a) {
        acc[2 * h + CHI * a] = df32(acc2[h][a].hi.x, acc2[h][a].lo.x);
        acc[2 * h + 1 + CHI * a] = df32(acc2[h][a].hi.y, acc2[h][a].lo.y);
      }
  } else {
    for (int f = tid; f < nfib; f += TEAM) {
      const int base = fiber_base(f);
      T x[CHI], y[CHI];
#pragma unroll
      for (int a = 0; a < CHI; ++a) {
        x[a] = t[spos<PAD>(base + a * st)];
        y[a] = conj_of(bra[spos<PAD>(base + bra_shift + a * st)]);
      }
#pragma unroll
      for (int a = 0; a < CHI; ++a)
#pragma unroll
        for (int b = 0; b < CHI; ++b) acc[b + CHI * a] = mac(y[b], x[a], acc[b + CHI * a]);
    }
  }
  const int lane = tid & 31, warp = tid >> 5;
  warp_reduce_scatter<T, P2>(acc, lane);
  // lane l now holds entries (l * PER, ...) for P2 >= 32; for P2 < 32 the top
  // log2(P2) lane bits select the entry and every lane of a group holds it
  constexpr int PER = P2 >= 32 ? P2 / 32 : 1;
  constexpr int SHIFT = P2 >= 32 ? 0 : (P2 == 1 ? 5 : P2 == 4 ? 3 : 1);
  const bool writer = (lane & ((1 << SHIFT) - 1)) == 0;
  const int first = P2 >= 32 ? lane * PER : (lane >> SHIFT);
  if constexpr (TEAM == 32) {
    if (writer) {
#pragma unroll
      for (int j = 0; j < PER; ++j) {
        const int o = first + j;
        if (o < P) res[o] = acc[j];
      }
    }
  } else {
    if (writer) {
#pragma unroll
      for (int j = 0; j < PER; ++j)
        if (first + j < P) red[warp * kRedStride + first + j] = acc[j];
    }
    __syncthreads();
    for (int o = tid; o < P; o += TEAM) {
      T s = T(0);
#pragma unroll
      for (int w = 0; w < TEAM / 32; ++w) s += red[w * kRedStride + o];
      res[o] = s;
    }
  }
  tsync<TEAM>();
}

template <typename T, int TEAM, bool PAD = false, bool PACK = false>
__device__ __forceinline__ void close_any(int chi, const T* t, const T* bra, int n, int st, int fib_mul,
                                          int fib_add, int bra_shift, T* red, T* res, int tid) {
  switch (chi) {
    case 1: close_fibers<T, 1, TEAM, PAD, PACK>(t, bra, n, st, fib_mul, fib_add, bra_shift, red, res, tid); break;
    case 2: close_fibers<T, 2, TEAM, PAD, PACK>(t, bra, n, st, fib_mul, fib_add, bra_shift, red, res, tid); break;
    case 3: close_fibers<T, 3, TEAM, PAD, PACK>(t, bra, n, st, fib_mul, fib_add, bra_shift, red, res, tid); break;
    case 4: close_fibers<T, 4, TEAM, PAD, PACK>(t, bra, n, st, fib_mul, fib_add, bra_shift, red, res, tid); break;
    case 5: close_fibers<T, 5, TEAM, PAD, PACK>(t, bra, n, st, fib_mul, fib_add, bra_shift, red, res, tid); break;
    case 6: close_fibers<T, 6, TEAM, PAD, PACK>(t, bra, n, st, fib_mul, fib_add, bra_shift, red, res, tid); break;
    case 7: close_fibers<T, 7, TEAM, PAD, PACK>(t, bra, n, st, fib_mul, fib_add, bra_shift, red, res, tid); break;
    case 8: close_fibers<T, 8, TEAM, PAD, PACK>(t, bra, n, st, fib_mul, fib_add, bra_shift, red, res, tid); break;
    default: break;
  }
}

// Normalise res (chi x chi) in FP64, write it to out, and (when diff != NULL)
// return message_diff(new, old) (abstractbeliefpropagationcache.jl:32-36) on
// lane 0.  Called by one full warp; old may alias out.
template <typename T>
__device__ __forceinline__ double finalize_message(const T* res, int chi, const T* old, T* out, int normalize,
                                                   bool want_diff, int lane) {
  const int P = chi * chi;
  const double v0 = lane < P ? (double)res[lane] : 0.0;
  const double v1 = lane + 32 < P ? (double)res[lane + 32] : 0.0;
  const double nrm2 = warp_sum(v0 * v0 + v1 * v1);
  const double sc = (normalize && nrm2 > 0.0) ? 1.0 / sqrt(nrm2) : 1.0;
  const T n0 = (T)(v0 * sc), n1 = (T)(v1 * sc);
  double o0 = 0.0, o1 = 0.0;
  if (want_diff) {
    if (lane < P) o0 = (double)old[lane];
    if (lane + 32 < P) o1 = (double)old[lane + 32];
  }
  __syncwarp();
  if (lane < P) out[lane] = n0;
  if (lane + 32 < P) out[lane + 32] = n1;
  double diff = 0.0;
  if (want_diff) {
    const double a0 = (double)n0, a1 = (double)n1;
    const double dot = warp_sum(a0 * o0 + a1 * o1);
    const double na = warp_sum(a0 * a0 + a1 * a1);
    const double nb = warp_sum(o0 * o0 + o1 * o1);
    diff = 1.0 - (dot * dot) / (na * nb);
  }
  return diff;
}

// Complex messages: Frobenius norm sum |x|^2, message_diff with the complex
// inner product <old, new> (|<a, b>|^2 as in the reference's message_diff).
template <>
__device__ __forceinline__ double finalize_message<zdouble>(const zdouble* res, int chi, const zdouble* old,
                                                            zdouble* out, int normalize, bool want_diff, int lane) {
  const int P = chi * chi;
  const zdouble v0 = lane < P ? res[lane] : zdouble(0.0), v1 = lane + 32 < P ? res[lane + 32] : zdouble(0.0);
  const double nrm2 = warp_sum(v0.re * v0.re + v0.im * v0.im + v1.re * v1.re + v1.im * v1.im);
  const double sc = (normalize && nrm2 > 0.0) ? 1.0 / sqrt(nrm2) : 1.0;
  const zdouble n0(v0.re * sc, v0.im * sc), n1(v1.re * sc, v1.im * sc);
  zdouble o0(0.0), o1(0.0);
  if (want_diff) {
    if (lane < P) o0 = old[lane];
    if (lane + 32 < P) o1 = old[lane + 32];
  }
  __syncwarp();
  if (lane < P) out[lane] = n0;
  if (lane + 32 < P) out[lane + 32] = n1;
  double diff = 0.0;
  if (want_diff) {
    // <o, n> = sum conj(o) n
    const double dre = warp_sum(o0.re * n0.re + o0.im * n0.im + o1.re * n1.re + o1.im * n1.im);
    const double dim = warp_sum(o0.re * n0.im - o0.im * n0.re + o1.re * n1.im - o1.im * n1.re);
    const double na = warp_sum(n0.re * n0.re + n0.im * n0.im + n1.re * n1.re + n1.im * n1.im);
    const double nb = warp_sum(o0.re * o0.re + o0.im * o0.im + o1.re * o1.re + o1.im * o1.im);
    diff = 1.0 - (dre * dre + dim * dim) / (na * nb);
  }
  return diff;
}

// Complex FP32 messages: as the complex FP64 case, with the norm, the scale
// and message_diff evaluated in FP64 and the result stored as FP32 pairs.
template <>
__device__ __forceinline__ double finalize_message<zfloat>(const zfloat* res, int chi, const zfloat* old, zfloat* out,
                                                           int normalize, bool want_diff, int lane) {
  const int P = chi * chi;
  const zfloat r0 = lane < P ? res[lane] : zfloat(0.f), r1 = lane + 32 < P ? res[lane + 32] : zfloat(0.f);
  const double v0r = r0.re, v0i = r0.im, v1r = r1.re, v1i = r1.im;
  const double nrm2 = warp_sum(v0r * v0r + v0i * v0i + v1r * v1r + v1i * v1i);
  const double sc = (normalize && nrm2 > 0.0) ? 1.0 / sqrt(nrm2) : 1.0;
  const zfloat n0((float)(v0r * sc), (float)(v0i * sc)), n1((float)(v1r * sc), (float)(v1i * sc));
  zfloat o0(0.f), o1(0.f);
  if (want_diff) {
    if (lane < P) o0 = old[lane];
    if (lane + 32 < P) o1 = old[lane + 32];
  }
  __syncwarp();
  if (lane < P) out[lane] = n0;
  if (lane + 32 < P) out[lane + 32] = n1;
  double diff = 0.0;
  if (want_diff) {
    const double a0r = n0.re, a0i = n0.im, a1r = n1.re, a1i = n1.im;
    const double b0r = o0.re, b0i = o0.im, b1r = o1.re, b1i = o1.im;
    const double dre = warp_sum(b0r * a0r + b0i * a0i + b1r * a1r + b1i * a1i);
    const double dim = warp_sum(b0r * a0i - b0i * a0r + b1r * a1i - b1i * a1r);
    const double na = warp_sum(a0r * a0r + a0i * a0i + a1r * a1r + a1i * a1i);
    const double nb = warp_sum(b0r * b0r + b0i * b0i + b1r * b1r + b1i * b1i);
    diff = 1.0 - (dre * dre + dim * dim) / (na * nb);
  }
  return diff;
}

// Double-FP32 arithmetic with FP64 storage: the result is formed in FP64
// (hi + lo), normalised and compared with the old FP64 message in FP64.
__device__ __forceinline__ double finalize_message_df(const df32* res, int chi, const double* old, double* out,
                                                      int normalize, bool want_diff, int lane) {
  const int P = chi * chi;
  const double v0 = lane < P ? df_to_double(res[lane]) : 0.0;
  const double v1 = lane + 32 < P ? df_to_double(res[lane + 32]) : 0.0;
  const double nrm2 = warp_sum(v0 * v0 + v1 * v1);
  const double sc = (normalize && nrm2 > 0.0) ? 1.0 / sqrt(nrm2) : 1.0;
  const double n0 = v0 * sc, n1 = v1 * sc;
  double o0 = 0.0, o1 = 0.0;
  if (want_diff) {
    if (lane < P) o0 = old[lane];
    if (lane + 32 < P) o1 = old[lane + 32];
  }
  __syncwarp();
  if (lane < P) out[lane] = n0;
  if (lane + 32 < P) out[lane + 32] = n1;
  double diff = 0.0;
  if (want_diff) {
    const double dot = warp_sum(n0 * o0 + n1 * o1);
    const double na = warp_sum(n0 * n0 + n1 * n1);
    const double nb = warp_sum(o0 * o0 + o1 * o1);
    diff = 1.0 - (dot * dot) / (na * nb);
  }
  return diff;
}

// Shared-memory carve-up of one team.  A team of several warps keeps one
// close result per leg (res: kMaxDeg x 64) and finalises them together after
// its last schedule step; a one-warp team finalises each as it is closed
// (res: 64).  old holds the previous outgoing messages (storage type, read by
// message_diff), loaded with the vertex so that no finalisation waits on HBM.
template <typename T>
struct TeamSmem {
  VDesc* desc;
  T* buf[kNumBufs];
  T* bra;
  T* msg;  // kMaxDeg x 64
  T* red;  // (TEAM/32) x kRedStride
  T* res;  // kMaxDeg x 64 (TEAM > 32) or 64
  T* old;  // kMaxDeg x 64 elements of T's size (holding the storage type)
};

__host__ __device__ inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

template <typename T>
__host__ __device__ inline size_t team_smem_bytes(int ncap, int nbuf, bool sep_bra, int team) {
  size_t b = align_up(sizeof(VDesc), 16);
  b += sizeof(T) * ((size_t)ncap * (nbuf + (sep_bra ? 1 : 0)) + team_tail_elems(team));
  return align_up(b, 16);
}

template <typename T>
__device__ __forceinline__ TeamSmem<T> carve(unsigned char* p, int ncap, int nbuf, bool sep_bra, int team) {
  TeamSmem<T> s;
  s.desc = reinterpret_cast<VDesc*>(p);
  T* q = reinterpret_cast<T*>(p + align_up(sizeof(VDesc), 16));
  for (int i = 0; i < kNumBufs; ++i) s.buf[i] = q + (size_t)ncap * (i < nbuf ? i : 0);
  q += (size_t)ncap * nbuf;
  if (sep_bra) {
    s.bra = q;
    q += ncap;
  } else {
    s.bra = s.buf[0];
  }
  s.msg = q;
  q += kMaxDeg * 64;
  s.red = q;
  q += (team / 32) * kRedStride;
  s.res = q;
  q += team > 32 ? kMaxDeg * 64 : 64;
  s.old = q;
  return s;
}

template <int TEAM>
__device__ __forceinline__ void load_desc(VDesc* dst, const VDesc* src, int tid) {
  constexpr int W = sizeof(VDesc) / 4;
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(dst);
  for (int i = tid; i < W; i += TEAM) d[i] = s[i];
}

// Load the tensor (and bra) of a vertex and its incoming messages (all legs,
// or all but skip_leg) into shared memory.
// S is the storage type in HBM (T, or double under df32 arithmetic).
template <typename T, int TEAM, typename S = T, bool PAD = false>
__device__ __forceinline__ void load_vertex(const TeamSmem<T>& Sm, const S* fac, const S* bra_g, const S* msgs,
                                            const long long* msg_off, int skip_leg, int tid) {
  const VDesc& d = *Sm.desc;
  const S* a = fac + d.a_off;
  // four loads in flight per thread before their stores
  int i = tid;
  for (; i + 3 * TEAM < d.n; i += 4 * TEAM) {
    const S x0 = a[i], x1 = a[i + TEAM], x2 = a[i + 2 * TEAM], x3 = a[i + 3 * TEAM];
    Sm.buf[0][spos<PAD>(i)] = to_elem<T>(x0);
    Sm.buf[0][spos<PAD>(i + TEAM)] = to_elem<T>(x1);
    Sm.buf[0][spos<PAD>(i + 2 * TEAM)] = to_elem<T>(x2);
    Sm.buf[0][spos<PAD>(i + 3 * TEAM)] = to_elem<T>(x3);
  }
  for (; i < d.n; i += TEAM) Sm.buf[0][spos<PAD>(i)] = to_elem<T>(a[i]);
  if (bra_g) {
    const S* b = bra_g + d.a_off;
    for (int i = tid; i < d.n; i += TEAM) Sm.bra[spos<PAD>(i)] = to_elem<T>(b[i]);
  }
  for (int p = 0; p < d.k; ++p) {
    if (p == skip_leg) continue;
    const int c2 = d.chi[p] * d.chi[p];
    const S* m = msgs + msg_off[d.in_de[p]];
    for (int i = tid; i < c2; i += TEAM) Sm.msg[p * 64 + i] = to_elem<T>(m[i]);
  }
}

// The current outgoing messages of a vertex (the "old" side of message_diff)
// into Sm.old, in their storage type.
template <typename T, int TEAM, typename S>
__device__ __forceinline__ void load_old_messages(const TeamSmem<T>& Sm, const S* msgs, const long long* msg_off,
                                                  int tid) {
  const VDesc& d = *Sm.desc;
  S* o = reinterpret_cast<S*>(Sm.old);
  for (int p = 0; p < d.k; ++p) {
    const int c2 = d.chi[p] * d.chi[p];
    const S* m = msgs + msg_off[d.out_de[p]];
    for (int i = tid; i < c2; i += TEAM) o[p * 64 + i] = m[i];
  }
}

}  // namespace gbtn
