// lh_fft.cuh -- batched mixed-radix (4, 3, 2) FFTs in shared memory.
//
// Replaces the FFTPACK-derived rfft/cfft kernels of the reference
// (rft_buff.f, cft_buff.f).  Every transform is an in-place decimation-in-
// frequency pass sequence over a batch of vectors held in shared memory; all
// threads of the CTA share the butterflies of a stage.  The output of a DIF
// sequence is in digit-reversed order; `perm[k]` gives the position of
// frequency (or sample) k.  Twiddles are tables of exp(-2 pi i k / n)
// computed on the host in extended precision, never evaluated on the device.
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
  int ns;                 // number of DIF stages
  int rad[kMaxStages];    // radix of stage s
  int len[kMaxStages];    // sub-transform length entering stage s (len[0] = n)
  const int* perm;        // device: position of index k after the DIF stages
  const double2* tw64;    // device: exp(-2 pi i k/n), k = 0..n-1
  const float2* tw32;     // same, rounded to float
};

template <typename R> __device__ __forceinline__ const cpx_t<R>* twtab(const FftPlan& p);
template <> __device__ __forceinline__ const double2* twtab<double>(const FftPlan& p) { return p.tw64; }
template <> __device__ __forceinline__ const float2* twtab<float>(const FftPlan& p) { return p.tw32; }

template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { return T2{a.x + b.x, a.y + b.y}; }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { return T2{a.x - b.x, a.y - b.y}; }
// a * w (SIGN < 0) or a * conj(w) (SIGN > 0), w from a table of exp(-i t)
template <int SIGN, typename T2> __device__ __forceinline__ T2 ctw(T2 a, T2 w) {
  if (SIGN < 0) return T2{a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x};
  return T2{a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y};
}

// In-place DIF over `nb` vectors: element e of vector b at buf[b*bs + e*es].
// SIGN = -1 forward (exp(-i)), +1 inverse (exp(+i)); no normalisation.
template <typename R, int SIGN>
__device__ void fft_dif(cpx_t<R>* buf, int nb, int es, int bs, const FftPlan& P) {
  using T2 = cpx_t<R>;
  const T2* __restrict__ tw = twtab<R>(P);
  const int n = P.n;
  for (int s = 0; s < P.ns; ++s) {
    const int r = P.rad[s], L = P.len[s], m = L / r, ts = n / L;
    const int nbf = n / r;
    const int total = nb * nbf;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int b = t / nbf, f = t - b * nbf;
      const int blk = f / m, k = f - blk * m;
      T2* base = buf + b * bs + (blk * L + k) * es;
      const int st = m * es;
      if (r == 4) {
        T2 a = base[0], bb = base[st], c = base[2 * st], d = base[3 * st];
        T2 t0 = cadd(a, c), t1 = csub(a, c), t2 = cadd(bb, d), t3 = csub(bb, d);
        // SIGN*i*t3
        T2 u = (SIGN < 0) ? T2{t3.y, -t3.x} : T2{-t3.y, t3.x};
        T2 y0 = cadd(t0, t2), y2 = csub(t0, t2), y1 = cadd(t1, u), y3 = csub(t1, u);
        if (m > 1) {
          y1 = ctw<SIGN>(y1, tw[k * ts]);
          y2 = ctw<SIGN>(y2, tw[2 * k * ts]);
          y3 = ctw<SIGN>(y3, tw[3 * k * ts]);
        }
        base[0] = y0; base[st] = y1; base[2 * st] = y2; base[3 * st] = y3;
      } else if (r == 2) {
        T2 a = base[0], bb = base[st];
        T2 y0 = cadd(a, bb), y1 = csub(a, bb);
        if (m > 1) y1 = ctw<SIGN>(y1, tw[k * ts]);
        base[0] = y0; base[st] = y1;
      } else {  // r == 3
        const R h = (R)0.5;
        const R s3 = (SIGN < 0) ? (R)-0.86602540378443864676 : (R)0.86602540378443864676;
        T2 a = base[0], bb = base[st], c = base[2 * st];
        T2 t1 = cadd(bb, c), d = csub(bb, c);
        T2 t2 = T2{a.x - h * t1.x, a.y - h * t1.y};
        T2 u = T2{-s3 * d.y, s3 * d.x};  // i*s3*d
        T2 y0 = cadd(a, t1), y1 = cadd(t2, u), y2 = csub(t2, u);
        if (m > 1) {
          y1 = ctw<SIGN>(y1, tw[k * ts]);
          y2 = ctw<SIGN>(y2, tw[2 * k * ts]);
        }
        base[0] = y0; base[st] = y1; base[2 * st] = y2;
      }
    }
    __syncthreads();
  }
}

}  // namespace lh
