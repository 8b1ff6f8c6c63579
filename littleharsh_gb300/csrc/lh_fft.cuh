// lh_fft.cuh -- batched mixed-radix (4, 2, 3) FFTs in shared memory.
//
// Replaces the FFTPACK-derived rfft/cfft kernels of the reference
// (rft_buff.f, cft_buff.f).  Every transform is an in-place decimation-in-
// time pass sequence over a batch of vectors held in shared memory; all
// threads of the CTA share the butterflies of a stage.  The input of a DIT
// sequence sits at digit-reversed positions (`perm[n]` is where sample n is
// stored) and the output comes out in natural order.  Twiddles are tables of
// exp(-2 pi i k / n) computed on the host in extended precision, never
// evaluated on the device.
//
// The butterflies are written for the FP64 pipe, which is the bottleneck on
// GB300 (1.2 TFLOP/s): each twiddle multiplication is fused into the
// butterfly's additions (a + w*c as two FMAs per component, a - w*c as
// 2a - (a + w*c)), so a radix-4 butterfly costs 24 FP64 instructions instead
// of 28, a radix-3 one 18 instead of 22 and a radix-2 one 6 instead of 8.
#pragma once
#include <cuda_runtime.h>

namespace lh {

template <typename R> struct cpx;
template <> struct cpx<double> { using T = double2; };
template <> struct cpx<float> { using T = float2; };
template <typename R> using cpx_t = typename cpx<R>::T;

constexpr int kMaxStages = 16;

// One transform length.  Passed by value to kernels.
struct FftPlan {
  int n;                  // length
  int ns;                 // number of DIT stages
  int rad[kMaxStages];    // radix of stage s (radix 4 first: stage 0 needs no twiddles; radix 3 last)
  int len[kMaxStages];    // transform length produced by stage s (len[ns-1] = n)
  int prune_mid;          // last stage is radix 3 over n/3 and the middle third of the output is not needed
  unsigned mdiv[kMaxStages];  // ceil(2^32 / (len[s] / rad[s])) (0 for 1): divides by a stage's butterfly span
  unsigned qdiv[kMaxStages];  // ceil(2^32 / (n / rad[s])) (0 for 1): divides by a stage's butterfly count
  const int* perm;        // device: position of sample n at the start (digit reversal)
  const double2* tw64;    // device: exp(-2 pi i k/n), k = 0..n-1
  const float2* tw32;     // same, rounded to float
};

template <typename R> __device__ __forceinline__ const cpx_t<R>* twtab(const FftPlan& p);
template <> __device__ __forceinline__ const double2* twtab<double>(const FftPlan& p) { return p.tw64; }
template <> __device__ __forceinline__ const float2* twtab<float>(const FftPlan& p) { return p.tw32; }

template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { return T2{a.x + b.x, a.y + b.y}; }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { return T2{a.x - b.x, a.y - b.y}; }

// b*w (SIGN < 0) or b*conj(w) (SIGN > 0), w from a table of exp(-i t): 2 instructions per component
template <int SIGN, typename T2> __device__ __forceinline__ T2 cmul(T2 b, T2 w) {
  if (SIGN < 0) return T2{fma(b.x, w.x, -(b.y * w.y)), fma(b.x, w.y, b.y * w.x)};
  return T2{fma(b.x, w.x, b.y * w.y), fma(b.y, w.x, -(b.x * w.y))};
}
// a + b*w (or a + b*conj(w)): two FMAs per component
template <int SIGN, typename T2> __device__ __forceinline__ T2 cmad(T2 a, T2 b, T2 w) {
  if (SIGN < 0) return T2{fma(b.x, w.x, fma(-b.y, w.y, a.x)), fma(b.x, w.y, fma(b.y, w.x, a.y))};
  return T2{fma(b.x, w.x, fma(b.y, w.y, a.x)), fma(b.y, w.x, fma(-b.x, w.y, a.y))};
}
// 2a - s: one FMA per component (the difference partner of s = a + x)
template <typename T2> __device__ __forceinline__ T2 ctwice_minus(T2 a, T2 s) {
  using R = decltype(a.x);
  return T2{fma((R)2, a.x, -s.x), fma((R)2, a.y, -s.y)};
}
// SIGN*i*t
template <int SIGN, typename T2> __device__ __forceinline__ T2 cimul(T2 t) {
  return (SIGN < 0) ? T2{t.y, -t.x} : T2{-t.y, t.x};
}

// One DIT butterfly of radix r at `base` (elements base[p*st], p = 0..r-1),
// twiddle exponent step e = k*(n/L) (0 for the first stage).
template <typename R, int SIGN>
__device__ __forceinline__ void dit_butterfly(cpx_t<R>* base, int st, int r, int e, bool twiddle, bool skip_mid,
                                              const cpx_t<R>* __restrict__ tw) {
  using T2 = cpx_t<R>;
  if (r == 4) {
    const T2 a = base[0], b = base[st], c = base[2 * st], d = base[3 * st];
    T2 t0, t1, t2, t3;
    if (twiddle) {
      const T2 w1 = tw[e], w2 = tw[2 * e], w3 = tw[3 * e];
      t0 = cmad<SIGN>(a, c, w2);
      t1 = ctwice_minus(a, t0);
      const T2 B = cmul<SIGN>(b, w1);
      t2 = cmad<SIGN>(B, d, w3);
      t3 = ctwice_minus(B, t2);
    } else {
      t0 = cadd(a, c); t1 = csub(a, c); t2 = cadd(b, d); t3 = csub(b, d);
    }
    const T2 u = cimul<SIGN>(t3);
    base[0] = cadd(t0, t2);
    base[st] = cadd(t1, u);
    base[2 * st] = csub(t0, t2);
    base[3 * st] = csub(t1, u);
  } else if (r == 2) {
    const T2 a = base[0], b = base[st];
    if (twiddle) {
      const T2 s = cmad<SIGN>(a, b, tw[e]);
      base[0] = s;
      base[st] = ctwice_minus(a, s);
    } else {
      base[0] = cadd(a, b);
      base[st] = csub(a, b);
    }
  } else {  // r == 3: X1 = a - t1/2 + SIGN*i*(sqrt3/2)(B - C), X2 its mirror
    const R s3 = (SIGN < 0) ? (R)-0.86602540378443864676 : (R)0.86602540378443864676;
    const T2 a = base[0], b = base[st], c = base[2 * st];
    T2 t1, d;
    if (twiddle) {
      const T2 B = cmul<SIGN>(b, tw[e]);
      t1 = cmad<SIGN>(B, c, tw[2 * e]);
      d = ctwice_minus(B, t1);
    } else {
      t1 = cadd(b, c);
      d = csub(b, c);
    }
    const T2 t2 = T2{fma((R)-0.5, t1.x, a.x), fma((R)-0.5, t1.y, a.y)};
    base[0] = cadd(a, t1);
    if (skip_mid) {
      base[2 * st] = T2{fma(s3, d.y, t2.x), fma(-s3, d.x, t2.y)};
    } else {
      const T2 x1 = T2{fma(-s3, d.y, t2.x), fma(s3, d.x, t2.y)};
      base[st] = x1;
      base[2 * st] = ctwice_minus(t2, x1);
    }
  }
}

// One DIT butterfly of radix RADIX on values held in registers (the same
// arithmetic as dit_butterfly); with skip_mid the radix-3 output v[1] is left
// as it was.
template <typename R, int SIGN, int RADIX>
__device__ __forceinline__ void bfly(cpx_t<R>* v, int e, bool twiddle, bool skip_mid,
                                     const cpx_t<R>* __restrict__ tw) {
  using T2 = cpx_t<R>;
  if constexpr (RADIX == 4) {
    const T2 a = v[0], b = v[1], c = v[2], d = v[3];
    T2 t0, t1, t2, t3;
    if (twiddle) {
      const T2 w1 = tw[e], w2 = tw[2 * e], w3 = tw[3 * e];
      t0 = cmad<SIGN>(a, c, w2);
      t1 = ctwice_minus(a, t0);
      const T2 B = cmul<SIGN>(b, w1);
      t2 = cmad<SIGN>(B, d, w3);
      t3 = ctwice_minus(B, t2);
    } else {
      t0 = cadd(a, c); t1 = csub(a, c); t2 = cadd(b, d); t3 = csub(b, d);
    }
    const T2 u = cimul<SIGN>(t3);
    v[0] = cadd(t0, t2);
    v[1] = cadd(t1, u);
    v[2] = csub(t0, t2);
    v[3] = csub(t1, u);
  } else if constexpr (RADIX == 2) {
    const T2 a = v[0], b = v[1];
    if (twiddle) {
      const T2 s = cmad<SIGN>(a, b, tw[e]);
      v[0] = s;
      v[1] = ctwice_minus(a, s);
    } else {
      v[0] = cadd(a, b);
      v[1] = csub(a, b);
    }
  } else {
    const R s3 = (SIGN < 0) ? (R)-0.86602540378443864676 : (R)0.86602540378443864676;
    const T2 a = v[0], b = v[1], c = v[2];
    T2 t1, d;
    if (twiddle) {
      const T2 B = cmul<SIGN>(b, tw[e]);
      t1 = cmad<SIGN>(B, c, tw[2 * e]);
      d = ctwice_minus(B, t1);
    } else {
      t1 = cadd(b, c);
      d = csub(b, c);
    }
    const T2 t2 = T2{fma((R)-0.5, t1.x, a.x), fma((R)-0.5, t1.y, a.y)};
    v[0] = cadd(a, t1);
    if (skip_mid) {
      v[2] = T2{fma(s3, d.y, t2.x), fma(-s3, d.x, t2.y)};
    } else {
      const T2 x1 = T2{fma(-s3, d.y, t2.x), fma(s3, d.x, t2.y)};
      v[1] = x1;
      v[2] = ctwice_minus(t2, x1);
    }
  }
}

// Shared-memory slot of element i of an x-transform buffer.  FP32 buffers
// hold one padding element after every 16: the digit-reversed input scatter
// and the first DIT stages step through the buffer in multiples of 4 and 16
// elements, which without padding meet in the same banks.  FP64 buffers are
// unpadded.
template <typename R> __device__ __forceinline__ int sxi(int i) {
  if constexpr (sizeof(R) == 4) return i + (i >> 4);
  else return i;
}
// elements to allocate for an x-transform buffer of n elements
template <typename R> __host__ __device__ constexpr size_t sx_elems(size_t n) {
  return sizeof(R) == 4 ? n + n / 16 + 1 : n;
}

// floor(t / d) for t * d < 2^32 as one multiply-high by mult = ceil(2^32 / d) (d > 1); d = 1 passes
// t through.  Exact: t (mult - 2^32 / d) / 2^32 < t / 2^32 < 1 / d, less than the gap between t / d and
// the next integer.
__host__ __device__ __forceinline__ unsigned fdiv_mult(unsigned d) {
  return d > 1 ? 0xFFFFFFFFu / d + 1u : 0u;  // = ceil(2^32 / d) for d > 1
}
__device__ __forceinline__ int fdiv(int t, int d, unsigned mult) {
  return d > 1 ? (int)__umulhi((unsigned)t, mult) : t;
}

// One DIT stage of radix RADIX over `nb` vectors (see fft_dit).
template <typename R, int SIGN, bool BFAST, int RADIX>
__device__ __forceinline__ void dit_stage(cpx_t<R>* buf, int nb, unsigned nbm, int es, int bs, int L, int n,
                                          unsigned mm, unsigned nbfm, bool skip_mid,
                                          const cpx_t<R>* __restrict__ tw) {
  const int m = L / RADIX, ts = n / L;
  const int nbf = n / RADIX;
  const int total = nb * nbf;
  const bool twiddle = m > 1;
  const int q = BFAST ? nb : nbf;  // the divisor that splits t into (vector, butterfly)
  const unsigned qm = BFAST ? nbm : nbfm;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int b, f;
    if (BFAST) { f = fdiv(t, q, qm); b = t - f * nb; }
    else { b = fdiv(t, q, qm); f = t - b * nbf; }
    const int blk = fdiv(f, m, mm), k = f - blk * m;
    cpx_t<R>* base = buf + b * bs + (blk * L + k) * es;
    dit_butterfly<R, SIGN>(base, m * es, RADIX, k * ts, twiddle, skip_mid, tw);
  }
}

// One DIT stage of radix RADIX over `nb` vectors of an FP32 x-transform buffer
// (es = 1, padded slots), index divisions as multiply-highs.
template <typename R, int SIGN, int RADIX>
__device__ __forceinline__ void dit_stage_padded(cpx_t<R>* buf, int nb, int bs, int L, int n, unsigned mm,
                                                 unsigned nbfm, bool skip_mid, const cpx_t<R>* __restrict__ tw) {
  const int m = L / RADIX, ts = n / L;
  const int nbf = n / RADIX;
  const int total = nb * nbf;
  const bool twiddle = m > 1;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int b = fdiv(t, nbf, nbfm), f = t - b * nbf;
    const int blk = fdiv(f, m, mm), k = f - blk * m;
    const int i0 = b * bs + blk * L + k;
    cpx_t<R> v[RADIX];
#pragma unroll
    for (int p = 0; p < RADIX; ++p) v[p] = buf[sxi<R>(i0 + p * m)];
    bfly<R, SIGN, RADIX>(v, k * ts, twiddle, skip_mid, tw);
#pragma unroll
    for (int p = 0; p < RADIX; ++p)
      if (!(RADIX == 3 && skip_mid && p == 1)) buf[sxi<R>(i0 + p * m)] = v[p];
  }
}

// Two FP32 x transforms in lockstep: element i of a float4 buffer holds sample i of one transform in (x, y)
// and of another in (z, w), in the padded slots of sxi<float>.  A thread runs the same butterfly of both with
// the arithmetic of dit_stage_padded, so each half comes out bit for bit as the one-transform path computes
// it, while the index arithmetic, the twiddle loads and the shared-memory instructions serve both.
__device__ __forceinline__ float2 lo2(float4 v) { return float2{v.x, v.y}; }
__device__ __forceinline__ float2 hi2(float4 v) { return float2{v.z, v.w}; }
__device__ __forceinline__ float4 cat4(float2 a, float2 b) { return float4{a.x, a.y, b.x, b.y}; }

template <int SIGN, int RADIX>
__device__ __forceinline__ void dit_stage_padded2(float4* buf, int nb, int bs, int L, int n, unsigned mm,
                                                  unsigned nbfm, const float2* __restrict__ tw) {
  const int m = L / RADIX, ts = n / L;
  const int nbf = n / RADIX;
  const int total = nb * nbf;
  const bool twiddle = m > 1;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int b = fdiv(t, nbf, nbfm), f = t - b * nbf;
    const int blk = fdiv(f, m, mm), k = f - blk * m;
    const int i0 = b * bs + blk * L + k;
    float2 va[RADIX], vb[RADIX];
#pragma unroll
    for (int p = 0; p < RADIX; ++p) {
      const float4 q = buf[sxi<float>(i0 + p * m)];
      va[p] = lo2(q);
      vb[p] = hi2(q);
    }
    bfly<float, SIGN, RADIX>(va, k * ts, twiddle, false, tw);
    bfly<float, SIGN, RADIX>(vb, k * ts, twiddle, false, tw);
#pragma unroll
    for (int p = 0; p < RADIX; ++p) buf[sxi<float>(i0 + p * m)] = cat4(va[p], vb[p]);
  }
}

// The DIT stages of plan P over nb float4 vectors (vector b at buf[b*bs]), input at digit-reversed positions.
template <int SIGN>
__device__ void fft_dit2(float4* buf, int nb, int bs, const FftPlan& P) {
  const float2* __restrict__ tw = P.tw32;
  const int n = P.n;
  for (int s = 0; s < P.ns; ++s) {
    const int r = P.rad[s], L = P.len[s];
    const unsigned mm = P.mdiv[s], nbfm = P.qdiv[s];
    if (r == 4) dit_stage_padded2<SIGN, 4>(buf, nb, bs, L, n, mm, nbfm, tw);
    else if (r == 2) dit_stage_padded2<SIGN, 2>(buf, nb, bs, L, n, mm, nbfm, tw);
    else dit_stage_padded2<SIGN, 3>(buf, nb, bs, L, n, mm, nbfm, tw);
    __syncthreads();
  }
}

// In-place DIT over `nb` vectors: element e of vector b at buf[b*bs + e*es].
// BFAST: consecutive threads take consecutive vectors (for interleaved
// vectors, es = nb-ish, bs = 1); otherwise consecutive butterflies of one
// vector (es = 1).  SIGN = -1 forward, +1 inverse; no normalisation.
// prune: skip the middle output third of the last radix-3 stage.
// FP32: the radix is resolved once per stage, so each stage's loop runs one
// butterfly form with its index divisions as multiply-highs; the FP32
// transforms are bound by instruction issue and shared memory, and this halves
// the integer work per butterfly.  FP32 x transforms (not BFAST; es = 1) use
// the padded slots of sxi.  FP64: one loop over all radices with plain divisions, which
// measures faster on the FP64 pipe, where the integer work runs alongside.
template <typename R, int SIGN, bool BFAST>
__device__ void fft_dit(cpx_t<R>* buf, int nb, int es, int bs, const FftPlan& P, bool prune) {
  using T2 = cpx_t<R>;
  const T2* __restrict__ tw = twtab<R>(P);
  const int n = P.n;
  if constexpr (sizeof(R) == 4) {
    const unsigned nbm = BFAST ? fdiv_mult((unsigned)nb) : 0u;
    for (int s = 0; s < P.ns; ++s) {
      const int r = P.rad[s], L = P.len[s];
      const unsigned mm = P.mdiv[s], nbfm = P.qdiv[s];
      const bool skip_mid = prune && s == P.ns - 1;
      if constexpr (BFAST) {
        if (r == 4) dit_stage<R, SIGN, BFAST, 4>(buf, nb, nbm, es, bs, L, n, mm, nbfm, false, tw);
        else if (r == 2) dit_stage<R, SIGN, BFAST, 2>(buf, nb, nbm, es, bs, L, n, mm, nbfm, false, tw);
        else dit_stage<R, SIGN, BFAST, 3>(buf, nb, nbm, es, bs, L, n, mm, nbfm, skip_mid, tw);
      } else {  // the x transforms: es = 1, padded buffer
        if (r == 4) dit_stage_padded<R, SIGN, 4>(buf, nb, bs, L, n, mm, nbfm, false, tw);
        else if (r == 2) dit_stage_padded<R, SIGN, 2>(buf, nb, bs, L, n, mm, nbfm, false, tw);
        else dit_stage_padded<R, SIGN, 3>(buf, nb, bs, L, n, mm, nbfm, skip_mid, tw);
      }
      __syncthreads();
    }
  } else {
    for (int s = 0; s < P.ns; ++s) {
      const int r = P.rad[s], L = P.len[s], m = L / r, ts = n / L;
      const int nbf = n / r;
      const int total = nb * nbf;
      const bool twiddle = m > 1;
      const bool skip_mid = prune && s == P.ns - 1;
      for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int b, f;
        if (BFAST) { f = t / nb; b = t - f * nb; }
        else { b = t / nbf; f = t - b * nbf; }
        const int blk = f / m, k = f - blk * m;
        T2* base = buf + b * bs + (blk * L + k) * es;
        dit_butterfly<R, SIGN>(base, m * es, r, k * ts, twiddle, skip_mid, tw);
      }
      __syncthreads();
    }
  }
}

}  // namespace lh
