// lh_kernels.cu -- sm_103a kernels of the Littleharsh RK3 substage.
//
// Data layout in HBM: every spectral field is plane-major complex
// [level][kk][i] (i = kx index fastest).  The reference moves y-pencils of one
// (kx,kz) column to x-z planes with MPI all-to-alls (FOU3D.f90, missing from
// the tree; call sites littleharsh.f90:171, tridLU_3D_IB.f90:220-245,302-324);
// here a plane kernel reads planes directly and a column kernel walks the
// levels of one column with coalesced per-level accesses, so no transpose
// pass exists in the step.
//
// Per substage:
//   zinv   z-inverse of u, w, v with 3/2 zero padding (the dk shift,
//          start.f90:1177-1205)                          -> mixed planes
//   xprod  x-inverse, y-interpolation to the other grid, the six products,
//          x-forward with truncation                      -> mixed products
//   zfwd   z-forward with truncation                      -> product spectra
//   assemble  RHS0_u1/2/3 (littleharsh.f90:614-731) + the reconstructed
//          nonlinear term + solveU/V's u+dt*du and the axz division
//          (tridLU_3D_IB.f90:90-98)
//   zinv/xmask/zfwd  canopy forcing on the processed planes
//          (immersed_boundaries_U/V, tridLU_3D_IB.f90:198-359)
//   vsolve Thomas sweeps with the shared y LU (tridLU_3D_IB.f90:106-116,179-189)
//   flowrate  meanflow_ctU/flowrate_corr on mode (0,0) (littleharsh.f90:453-485)
//   psolve divergence, pressure LU per column, p += psi, v_corr
//          (littleharsh.f90:557-612,826-937; tridLU_3D_IB.f90:362-396)
#include <algorithm>
#include <cstdio>

#include "lh_internal.h"

namespace lh {

// ---------------------------------------------------------------------------
// z passes
// ---------------------------------------------------------------------------

template <typename R>
__device__ __forceinline__ void zinv_body(const ZJobs<R>& jobs, const Dims& d, const FftPlan& pz, int tx, int bx,
                                          int by, int bz) {
  using T2 = cpx_t<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  T2* sm = reinterpret_cast<T2*>(smraw);  // [ngz][tx]
  const int job = bz;
  const ZJob<R> J = jobs.j[job];
  const int y = by;
  if (y >= J.nlev) return;
  const int lev = J.levels ? J.levels[y] : J.lev0 + y;
  const int i0 = bx * tx;
  const int nb = min(tx, d.nkx - i0);
  const double2* __restrict__ src = J.spec_in + (size_t)lev * d.np;
  const int h = d.nz / 2, gap = d.ngz - d.nz;
  // samples go to their digit-reversed positions; the 3/2 padding slots are zero
  for (int e = threadIdx.x; e < gap * tx; e += blockDim.x) sm[pz.perm[h + e / tx] * tx + (e % tx)] = T2{0, 0};
  for (int e = threadIdx.x; e < d.nz * tx; e += blockDim.x) {
    const int kk = e / tx, c = e - kk * tx;
    const int slot = kk < h ? kk : kk + gap;
    T2 v = T2{0, 0};
    if (c < nb && !(J.nomean && kk == 0 && i0 + c == 0)) {
      const int ks = kk < h ? kk : kk - d.nz + d.snz;  // row of the stored mode set
      const double2 s = src[(size_t)ks * d.spitch + i0 + c];
      v = T2{(R)s.x, (R)s.y};
    }
    sm[pz.perm[slot] * tx + c] = v;
  }
  __syncthreads();
  fft_dit<R, +1, true>(sm, nb, tx, 1, pz, false);
  T2* __restrict__ dst = J.mix + (size_t)y * d.mp;
  for (int e = threadIdx.x; e < d.ngz * tx; e += blockDim.x) {
    const int z = e / tx, c = e - z * tx;
    if (c < nb) dst[(size_t)z * d.nkx + i0 + c] = sm[z * tx + c];
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_zinv(const __grid_constant__ ZJobs<R> jobs, const __grid_constant__ Dims d,
                                              const __grid_constant__ FftPlan pz, int tx) {
  zinv_body<R>(jobs, d, pz, tx, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <typename R>
__device__ __forceinline__ void zfwd_body(const ZJobs<R>& jobs, const Dims& d, const FftPlan& pz, int tx, double scale,
                                          int bx, int by, int bz) {
  using T2 = cpx_t<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  T2* sm = reinterpret_cast<T2*>(smraw);  // [ngz][tx]
  const int job = bz;
  const ZJob<R> J = jobs.j[job];
  const int y = by;
  if (y >= J.nlev) return;
  const int lev = J.levels ? J.levels[y] : J.lev0 + y;
  const int i0 = bx * tx;
  const int nb = min(tx, d.nkx - i0);
  const T2* __restrict__ src = J.mix + (size_t)y * d.mp;
  for (int e = threadIdx.x; e < d.ngz * tx; e += blockDim.x) {
    const int z = e / tx, c = e - z * tx;
    sm[pz.perm[z] * tx + c] = (c < nb) ? src[(size_t)z * d.nkx + i0 + c] : T2{0, 0};
  }
  __syncthreads();
  // the truncation keeps slots [0, N2/2) and [Ngz - N2/2, Ngz): the middle third of the last radix-3
  // stage's output is never read when N2/2 = Ngz/3
  fft_dit<R, -1, true>(sm, nb, tx, 1, pz, pz.prune_mid != 0);
  const int h = d.nz / 2, gap = d.ngz - d.nz;
  if constexpr (sizeof(R) == 4) {
    if (J.out32) {  // the mixed form's product spectra stay FP32 (only the nonlinear term reads them)
      T2* __restrict__ dst = reinterpret_cast<T2*>(J.spec_out) + (size_t)lev * d.np;
      const R sc = (R)scale;
      for (int e = threadIdx.x; e < d.nz * tx; e += blockDim.x) {
        const int kk = e / tx, c = e - kk * tx;
        if (c < nb) {
          const int slot = kk < h ? kk : kk + gap;
          const T2 v = sm[slot * tx + c];
          const int ks = kk < h ? kk : kk - d.nz + d.snz;
          dst[(size_t)ks * d.spitch + i0 + c] = T2{v.x * sc, v.y * sc};
        }
      }
      return;
    }
  }
  double2* __restrict__ dst = J.spec_out + (size_t)lev * d.np;
  for (int e = threadIdx.x; e < d.nz * tx; e += blockDim.x) {
    const int kk = e / tx, c = e - kk * tx;
    if (c < nb) {
      const int slot = kk < h ? kk : kk + gap;
      const T2 v = sm[slot * tx + c];
      const int ks = kk < h ? kk : kk - d.nz + d.snz;
      dst[(size_t)ks * d.spitch + i0 + c] = double2{(double)v.x * scale, (double)v.y * scale};
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_zfwd(const __grid_constant__ ZJobs<R> jobs, const __grid_constant__ Dims d,
                                              const __grid_constant__ FftPlan pz, int tx, double scale) {
  zfwd_body<R>(jobs, d, pz, tx, scale, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <typename R>
void zpass_shape(const ZJobs<R>& jobs, const Dims& d, int tx, dim3* grid, size_t* smem) {
  *grid = (jobs.njobs == 0 || jobs.maxlev == 0) ? dim3(0, 0, 0) : dim3((d.nkx + tx - 1) / tx, jobs.maxlev, jobs.njobs);
  *smem = sizeof(cpx_t<R>) * (size_t)d.ngz * tx;
}

template <typename R>
void launch_zinv(const ZJobs<R>& jobs, const Dims& d, const FftPlan& pz, int tx, cudaStream_t st, int threads) {
  dim3 grid;
  size_t sm;
  zpass_shape(jobs, d, tx, &grid, &sm);
  if (grid.x == 0) return;
  k_zinv<R><<<grid, threads == 128 ? 128 : 256, sm, st>>>(jobs, d, pz, tx);
}

template <typename R>
void launch_zfwd(const ZJobs<R>& jobs, const Dims& d, const FftPlan& pz, int tx, double scale, cudaStream_t st,
                 int threads) {
  dim3 grid;
  size_t sm;
  zpass_shape(jobs, d, tx, &grid, &sm);
  if (grid.x == 0) return;
  k_zfwd<R><<<grid, threads == 128 ? 128 : 256, sm, st>>>(jobs, d, pz, tx, scale);
}

// ---------------------------------------------------------------------------
// x passes: real transforms of length ngx through complex DIFs of length h = ngx/2
// ---------------------------------------------------------------------------

// Inverse real transform of `nr` mixed rows (nkx complex each, zero beyond)
// into physical rows (ngx reals).  F: nr vectors of hp complex.
template <typename R>
__device__ void x_inverse(const cpx_t<R>* const* rows, int nr, cpx_t<R>* F, int hp, R* const* out, const Dims& d,
                          const FftPlan& ph, const double2* __restrict__ rtw) {
  using T2 = cpx_t<R>;
  const int h = d.ngx / 2, nkx = d.nkx;
  for (int e = threadIdx.x; e < nr * h; e += blockDim.x) {
    const int r = e / h, k = e - r * h;
    const T2* row = rows[r];
    T2 a = (k < nkx) ? row[k] : T2{0, 0};
    if (k == 0) a.y = 0;
    const int k2 = h - k;  // k = 0 pairs with X[h] = 0
    T2 b = (k > 0 && k2 < nkx) ? row[k2] : T2{0, 0};
    b.y = -b.y;
    const T2 s = cadd(a, b), df = csub(a, b);
    const double2 w = rtw[k];
    const R wr = (R)w.x, wi = (R)-w.y;  // exp(+2 pi i k/n)
    const T2 q = T2{wr * df.x - wi * df.y, wr * df.y + wi * df.x};
    F[sxi<R>(r * hp + ph.perm[k])] = T2{s.x - q.y, s.y + q.x};
  }
  __syncthreads();
  fft_dit<R, +1, false>(F, nr, 1, hp, ph, false);
  for (int e = threadIdx.x; e < nr * h; e += blockDim.x) {
    const int r = e / h, m = e - r * h;
    const T2 z = F[sxi<R>(r * hp + m)];
    out[r][2 * m] = z.x;
    out[r][2 * m + 1] = z.y;
  }
  __syncthreads();
}

// Forward real transform of the data already packed in F (z[m] = x[2m] + i
// x[2m+1] stored at position perm[m]) into nr mixed rows scaled by 1/ngx,
// kx < nkx kept.
template <typename R>
__device__ void x_forward_packed(int nr, cpx_t<R>* F, int hp, cpx_t<R>* const* rows, const Dims& d,
                                 const FftPlan& ph, const double2* __restrict__ rtw) {
  using T2 = cpx_t<R>;
  const int h = d.ngx / 2, nkx = d.nkx;
  const R scale = (R)(1.0 / d.ngx);
  fft_dit<R, -1, false>(F, nr, 1, hp, ph, false);
  for (int e = threadIdx.x; e < nr * nkx; e += blockDim.x) {
    const int r = e / nkx, k = e - r * nkx;
    const T2 zk = F[sxi<R>(r * hp + k)];
    const int k2 = (h - k) % h;
    T2 zc = F[sxi<R>(r * hp + k2)];
    zc.y = -zc.y;
    const T2 E = T2{(R)0.5 * (zk.x + zc.x), (R)0.5 * (zk.y + zc.y)};
    const T2 D = csub(zk, zc);
    const T2 O = T2{(R)0.5 * D.y, (R)-0.5 * D.x};
    const double2 w = rtw[k];
    const R wr = (R)w.x, wi = (R)w.y;
    T2 X = T2{E.x + (wr * O.x - wi * O.y), E.y + (wr * O.y + wi * O.x)};
    X.x = scale * X.x;
    X.y = (k == 0) ? (R)0 : scale * X.y;
    rows[r][k] = X;
  }
  __syncthreads();
}

// Two real rows through one complex transform of length ngx (n): the inverse
// takes the mixed rows A, B (nkx modes, zero beyond, imaginary part of the
// kx = 0 mode dropped as the real inverse does) as z = a + i b; the forward
// splits the transform of z = a + i b into the two half spectra.  This costs
// fewer FP64 instructions than two half-length real transforms with their
// pre/post twiddle passes.
template <typename R>
__device__ void x_inverse_pair(const cpx_t<R>* rowA, const cpx_t<R>* rowB, cpx_t<R>* F, R* outA, R* outB,
                               const Dims& d, const FftPlan& pf) {
  using T2 = cpx_t<R>;
  const int n = d.ngx, nkx = d.nkx;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    T2 z = T2{0, 0};
    if (k == 0) {
      z = T2{rowA[0].x, rowB[0].x};
    } else if (k < nkx) {
      const T2 a = rowA[k], b = rowB[k];
      z = T2{a.x - b.y, a.y + b.x};
    } else if (k > n - nkx) {
      const T2 a = rowA[n - k], b = rowB[n - k];
      z = T2{a.x + b.y, b.x - a.y};
    }
    F[sxi<R>(pf.perm[k])] = z;
  }
  __syncthreads();
  fft_dit<R, +1, false>(F, 1, 1, n, pf, false);
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    const T2 z = F[sxi<R>(x)];
    outA[x] = z.x;
    outB[x] = z.y;
  }
  __syncthreads();
}

// Forward transform of np2 packed pairs F[p*n + perm[x]] = a[x] + i b[x]
// into 2*np2 mixed rows (kx < nkx, scaled by 1/ngx).
template <typename R>
__device__ void x_forward_pairs(int np2, cpx_t<R>* F, cpx_t<R>* const* rows, const Dims& d, const FftPlan& pf) {
  using T2 = cpx_t<R>;
  const int n = d.ngx, nkx = d.nkx;
  const R sc = (R)(0.5 / n);
  fft_dit<R, -1, false>(F, np2, 1, n, pf, false);
  for (int e = threadIdx.x; e < np2 * nkx; e += blockDim.x) {
    const int p = e / nkx, k = e - p * nkx;
    const T2 zk = F[sxi<R>(p * n + k)];
    const T2 zc = F[sxi<R>(p * n + ((n - k) % n))];
    rows[2 * p][k] = T2{sc * (zk.x + zc.x), sc * (zk.y - zc.y)};
    rows[2 * p + 1][k] = T2{sc * (zk.y + zc.y), sc * (zc.x - zk.x)};
  }
  __syncthreads();
}

template <typename R>
__device__ __forceinline__ void xprod_body(const ProdArgs<R>& a, const Dims& d, const FftPlan& ph, const FftPlan& pf,
                                           const double2* __restrict__ rtw, int bx, int by) {
  using T2 = cpx_t<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ngx = d.ngx, h = ngx / 2, hp = h + 1;
  // 3 vectors of ngx, 2 with a.split (also holds the half-length v transform)
  T2* F = reinterpret_cast<T2*>(smraw);
  R* rowsm = reinterpret_cast<R*>(F + sx_elems<R>((a.split ? 2 : 3) * (size_t)ngx));  // 6 rows of ngx
  R* up = rowsm;
  R* wp = rowsm + ngx;
  R* vp = rowsm + 2 * ngx;
  R* uc = rowsm + 3 * ngx;
  R* wc = rowsm + 4 * ngx;
  R* vc = rowsm + 5 * ngx;
  __shared__ double cflred[8];
  const int kz = bx;
  // step jj forms the centre-jj products (c_lo <= jj <= c_hi) and the face-(jj-1) ones (f_lo <= jj-1 <= f_hi)
  const int L0 = min(a.c_lo, a.f_lo + 1), L1 = max(a.c_hi, a.f_hi + 1);
  const int c0 = L0 + by * a.chunk;
  const int c1 = min(c0 + a.chunk - 1, L1);
  if (c0 > c1) return;
  const size_t rowoff = (size_t)kz * d.nkx;
  double cmax = 0.0;
  // warm-up: previous centre and face
  if (c0 - 1 >= 1) {
    x_inverse_pair<R>(a.mu + (size_t)(c0 - 1) * d.mp + rowoff, a.mw + (size_t)(c0 - 1) * d.mp + rowoff, F, up, wp, d,
                      pf);
    const T2* rows[1] = {a.mv + (size_t)(c0 - 1) * d.mp + rowoff};
    R* outs[1] = {vp};
    x_inverse<R>(rows, 1, F, hp, outs, d, ph, rtw);
  } else {
    for (int x = threadIdx.x; x < 3 * ngx; x += blockDim.x) up[x] = (R)0;
    __syncthreads();
  }
  for (int jj = c0; jj <= c1; ++jj) {
    const bool vface = jj <= d.nyv - 2;  // face jj interior (else the top wall, v = 0)
    x_inverse_pair<R>(a.mu + (size_t)jj * d.mp + rowoff, a.mw + (size_t)jj * d.mp + rowoff, F, uc, wc, d, pf);
    if (vface) {
      const T2* rows[1] = {a.mv + (size_t)jj * d.mp + rowoff};
      R* outs[1] = {vc};
      x_inverse<R>(rows, 1, F, hp, outs, d, ph, rtw);
    } else {
      for (int x = threadIdx.x; x < ngx; x += blockDim.x) vc[x] = (R)0;
      __syncthreads();
    }
    const bool cprod = jj >= a.c_lo && jj <= a.c_hi;
    const bool fprod = jj - 1 >= a.f_lo && jj - 1 <= a.f_hi;  // face jj-1 interior and in this launch
    const R wcj = (R)a.wc[jj];
    const R wfj = fprod ? (R)a.wf[jj - 1] : (R)0;
    const double dyi = a.dyc[jj];
    // pairs: (uu, uw), (ww, vv) at centre jj; (uv, vw) at face jj-1 (after the centre pairs, or first);
    // with a.split and both kinds, the face pair goes through the buffer after the centre pairs' transform
    const bool later = a.split && cprod && fprod;
    const int fslot = (cprod && !later) ? 2 : 0;
    // mixed form: the level means at centre jj and face jj-1 (the FP64 form transforms u and w whole)
    R Uc = (R)0, Wc = (R)0, Uf = (R)0, Wf = (R)0;
    if constexpr (sizeof(R) == 4) {
      if (a.mean_split) {
        const R Um = (R)a.us[(size_t)(jj - 1) * a.nps].x, Wm = (R)a.ws[(size_t)(jj - 1) * a.nps].x;
        Uc = (R)a.us[(size_t)jj * a.nps].x;
        Wc = (R)a.ws[(size_t)jj * a.nps].x;
        Uf = Um + wfj * (Uc - Um);
        Wf = Wm + wfj * (Wc - Wm);
      }
    }
    auto face_pair = [&](int x, R u, R w, int px) {
      const R uf = up[x] + wfj * (u - up[x]);
      const R wf = wp[x] + wfj * (w - wp[x]);
      if constexpr (sizeof(R) == 4) F[sxi<R>(fslot * ngx + px)] = T2{(Uf + uf) * vp[x], (Wf + wf) * vp[x]};
      else F[sxi<R>(fslot * ngx + px)] = T2{uf * vp[x], wf * vp[x]};
    };
    for (int x = threadIdx.x; x < ngx; x += blockDim.x) {
      const R u = uc[x], w = wc[x];
      const int px = pf.perm[x];
      if (cprod) {
        const R v = vp[x] + wcj * (vc[x] - vp[x]);
        if constexpr (sizeof(R) == 4) {
          F[sxi<R>(px)] = T2{u * ((Uc + Uc) + u), u * (Wc + w) + Uc * w};
          F[sxi<R>(ngx + px)] = T2{w * ((Wc + Wc) + w), v * v};
        } else {
          F[sxi<R>(px)] = T2{u * u, u * w};
          F[sxi<R>(ngx + px)] = T2{w * w, v * v};
        }
        if (a.want_cfl) {
          const double cv = fabs((double)u) * a.dxi + fabs((double)v) * dyi + fabs((double)w) * a.dzi;
          cmax = fmax(cmax, cv);
        }
      }
      if (fprod && !later) face_pair(x, u, w, px);
    }
    __syncthreads();
    if (cprod || fprod) {
      T2* rows[6];
      int npair = 0;
      if (cprod) {
        for (int q = 0; q < 4; ++q) rows[q] = a.out[q] + (size_t)jj * d.mp + rowoff;
        npair = 2;
      }
      if (fprod) {
        rows[2 * npair] = a.out[4] + (size_t)(jj - 1) * d.mp + rowoff;
        rows[2 * npair + 1] = a.out[5] + (size_t)(jj - 1) * d.mp + rowoff;
        ++npair;
      }
      if (later) {
        x_forward_pairs<R>(2, F, rows, d, pf);
        for (int x = threadIdx.x; x < ngx; x += blockDim.x) face_pair(x, uc[x], wc[x], pf.perm[x]);
        __syncthreads();
        x_forward_pairs<R>(1, F, rows + 4, d, pf);
      } else {
        x_forward_pairs<R>(npair, F, rows, d, pf);
      }
    }
    // current becomes previous
    R* t;
    t = up; up = uc; uc = t;
    t = wp; wp = wc; wc = t;
    t = vp; vp = vc; vc = t;
  }
  if (a.want_cfl) {
    for (int o = 16; o > 0; o >>= 1) cmax = fmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
    if ((threadIdx.x & 31) == 0) cflred[threadIdx.x >> 5] = cmax;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, cflred[w]);
      atomicMax(&a.sc->cflbits, (unsigned long long)__double_as_longlong(m));
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_xprod(const __grid_constant__ ProdArgs<R> a, const __grid_constant__ Dims d,
                                               const __grid_constant__ FftPlan ph, const __grid_constant__ FftPlan pf,
                                               const double2* __restrict__ rtw) {
  xprod_body<R>(a, d, ph, pf, rtw, blockIdx.x, blockIdx.y);
}

// ---- the FP32 product pass on two z rows per CTA --------------------------------------------------------
// The same work as xprod_body for the rows 2 bx and 2 bx + 1, their transforms run in lockstep (fft_dit2):
// element x of a float4 transform buffer holds row 0's complex sample in (x, y) and row 1's in (z, w), and a
// physical row keeps both rows' values as float2 pairs.  Every per-row operation is the one xprod_body does,
// in the same order, so the results are the same bit for bit; the index arithmetic, twiddle and permutation
// loads and shared-memory instructions of a butterfly or an element serve both rows.

// xprod_body's x_inverse_pair for two rows: z = a + i b of row q in the q-th half of each element
__device__ void x_inverse_pair2(const float2* rowA0, const float2* rowB0, const float2* rowA1, const float2* rowB1,
                                float4* F, float2* outA, float2* outB, const Dims& d, const FftPlan& pf) {
  const int n = d.ngx, nkx = d.nkx;
  auto pack = [&](const float2* rowA, const float2* rowB, int k) {
    float2 z = float2{0.f, 0.f};
    if (k == 0) {
      z = float2{rowA[0].x, rowB[0].x};
    } else if (k < nkx) {
      const float2 a = rowA[k], b = rowB[k];
      z = float2{a.x - b.y, a.y + b.x};
    } else if (k > n - nkx) {
      const float2 a = rowA[n - k], b = rowB[n - k];
      z = float2{a.x + b.y, b.x - a.y};
    }
    return z;
  };
  for (int k = threadIdx.x; k < n; k += blockDim.x)
    F[sxi<float>(pf.perm[k])] = cat4(pack(rowA0, rowB0, k), pack(rowA1, rowB1, k));
  __syncthreads();
  fft_dit2<+1>(F, 1, n, pf);
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    const float4 z = F[sxi<float>(x)];
    outA[x] = float2{z.x, z.z};
    outB[x] = float2{z.y, z.w};
  }
  __syncthreads();
}

// xprod_body's half-length inverse of one v row, for two rows
__device__ void x_inverse2(const float2* row0, const float2* row1, float4* F, float2* out, const Dims& d,
                           const FftPlan& ph, const double2* __restrict__ rtw) {
  const int h = d.ngx / 2, nkx = d.nkx;
  auto pre = [&](const float2* row, int k, float wr, float wi) {
    float2 a = (k < nkx) ? row[k] : float2{0.f, 0.f};
    if (k == 0) a.y = 0.f;
    const int k2 = h - k;
    float2 b = (k > 0 && k2 < nkx) ? row[k2] : float2{0.f, 0.f};
    b.y = -b.y;
    const float2 s = cadd(a, b), df = csub(a, b);
    const float2 q = float2{wr * df.x - wi * df.y, wr * df.y + wi * df.x};
    return float2{s.x - q.y, s.y + q.x};
  };
  for (int k = threadIdx.x; k < h; k += blockDim.x) {
    const double2 w = rtw[k];
    const float wr = (float)w.x, wi = (float)-w.y;  // exp(+2 pi i k/n)
    F[sxi<float>(ph.perm[k])] = cat4(pre(row0, k, wr, wi), pre(row1, k, wr, wi));
  }
  __syncthreads();
  fft_dit2<+1>(F, 1, h + 1, ph);
  for (int m = threadIdx.x; m < h; m += blockDim.x) {
    const float4 z = F[sxi<float>(m)];
    out[2 * m] = float2{z.x, z.z};
    out[2 * m + 1] = float2{z.y, z.w};
  }
  __syncthreads();
}

// xprod_body's x_forward_pairs for two rows: np2 packed pairs into rows0[2p], rows0[2p+1] (row 0) and
// rows1[2p], rows1[2p+1] (row 1)
__device__ void x_forward_pairs2(int np2, float4* F, float2* const* rows0, float2* const* rows1, const Dims& d,
                                 const FftPlan& pf) {
  const int n = d.ngx, nkx = d.nkx;
  const float sc = (float)(0.5 / n);
  fft_dit2<-1>(F, np2, n, pf);
  for (int e = threadIdx.x; e < np2 * nkx; e += blockDim.x) {
    const int p = e / nkx, k = e - p * nkx;
    const float4 zk4 = F[sxi<float>(p * n + k)];
    const float4 zc4 = F[sxi<float>(p * n + ((n - k) % n))];
    const float2 zk0 = lo2(zk4), zc0 = lo2(zc4), zk1 = hi2(zk4), zc1 = hi2(zc4);
    rows0[2 * p][k] = float2{sc * (zk0.x + zc0.x), sc * (zk0.y - zc0.y)};
    rows0[2 * p + 1][k] = float2{sc * (zk0.y + zc0.y), sc * (zc0.x - zk0.x)};
    rows1[2 * p][k] = float2{sc * (zk1.x + zc1.x), sc * (zk1.y - zc1.y)};
    rows1[2 * p + 1][k] = float2{sc * (zk1.y + zc1.y), sc * (zc1.x - zk1.x)};
  }
  __syncthreads();
}

__device__ __forceinline__ void xprod2_body(const ProdArgs<float>& a, const Dims& d, const FftPlan& ph,
                                            const FftPlan& pf, const double2* __restrict__ rtw, int bx, int by) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ngx = d.ngx;
  float4* F = reinterpret_cast<float4*>(smraw);  // 3 vectors of ngx
  float2* rowsm = reinterpret_cast<float2*>(F + sx_elems<float>(3 * (size_t)ngx));  // 6 rows of ngx pairs
  float2* up = rowsm;
  float2* wp = rowsm + ngx;
  float2* vp = rowsm + 2 * ngx;
  float2* uc = rowsm + 3 * ngx;
  float2* wc = rowsm + 4 * ngx;
  float2* vc = rowsm + 5 * ngx;
  __shared__ double cflred[8];
  const int kz0 = 2 * bx;
  const int L0 = min(a.c_lo, a.f_lo + 1), L1 = max(a.c_hi, a.f_hi + 1);
  const int c0 = L0 + by * a.chunk;
  const int c1 = min(c0 + a.chunk - 1, L1);
  if (c0 > c1) return;
  const size_t ro0 = (size_t)kz0 * d.nkx, ro1 = ro0 + d.nkx;
  double cmax = 0.0;
  auto inverse = [&](int lev, float2* ou, float2* ow) {
    const size_t o = (size_t)lev * d.mp;
    x_inverse_pair2(a.mu + o + ro0, a.mw + o + ro0, a.mu + o + ro1, a.mw + o + ro1, F, ou, ow, d, pf);
  };
  if (c0 - 1 >= 1) {
    inverse(c0 - 1, up, wp);
    const size_t o = (size_t)(c0 - 1) * d.mp;
    x_inverse2(a.mv + o + ro0, a.mv + o + ro1, F, vp, d, ph, rtw);
  } else {
    for (int x = threadIdx.x; x < 3 * ngx; x += blockDim.x) up[x] = float2{0.f, 0.f};
    __syncthreads();
  }
  for (int jj = c0; jj <= c1; ++jj) {
    const bool vface = jj <= d.nyv - 2;
    inverse(jj, uc, wc);
    if (vface) {
      const size_t o = (size_t)jj * d.mp;
      x_inverse2(a.mv + o + ro0, a.mv + o + ro1, F, vc, d, ph, rtw);
    } else {
      for (int x = threadIdx.x; x < ngx; x += blockDim.x) vc[x] = float2{0.f, 0.f};
      __syncthreads();
    }
    const bool cprod = jj >= a.c_lo && jj <= a.c_hi;
    const bool fprod = jj - 1 >= a.f_lo && jj - 1 <= a.f_hi;
    const float wcj = (float)a.wc[jj];
    const float wfj = fprod ? (float)a.wf[jj - 1] : 0.f;
    const double dyi = a.dyc[jj];
    const int fslot = cprod ? 2 : 0;
    float Uc = 0.f, Wc = 0.f, Uf = 0.f, Wf = 0.f;
    if (a.mean_split) {
      const float Um = (float)a.us[(size_t)(jj - 1) * a.nps].x, Wm = (float)a.ws[(size_t)(jj - 1) * a.nps].x;
      Uc = (float)a.us[(size_t)jj * a.nps].x;
      Wc = (float)a.ws[(size_t)jj * a.nps].x;
      Uf = Um + wfj * (Uc - Um);
      Wf = Wm + wfj * (Wc - Wm);
    }
    for (int x = threadIdx.x; x < ngx; x += blockDim.x) {
      const float2 u2 = uc[x], w2 = wc[x];
      const int px = pf.perm[x];
      const float us[2] = {u2.x, u2.y}, ws[2] = {w2.x, w2.y};
      if (cprod) {
        const float2 vp2 = vp[x], vc2 = vc[x];
        const float vps[2] = {vp2.x, vp2.y}, vcs[2] = {vc2.x, vc2.y};
        float2 p0[2], p1[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float u = us[q], w = ws[q];
          const float v = vps[q] + wcj * (vcs[q] - vps[q]);
          p0[q] = float2{u * ((Uc + Uc) + u), u * (Wc + w) + Uc * w};
          p1[q] = float2{w * ((Wc + Wc) + w), v * v};
          if (a.want_cfl) {
            const double cv = fabs((double)u) * a.dxi + fabs((double)v) * dyi + fabs((double)w) * a.dzi;
            cmax = fmax(cmax, cv);
          }
        }
        F[sxi<float>(px)] = cat4(p0[0], p0[1]);
        F[sxi<float>(ngx + px)] = cat4(p1[0], p1[1]);
      }
      if (fprod) {
        const float2 up2 = up[x], wp2 = wp[x], vp2 = vp[x];
        const float ups[2] = {up2.x, up2.y}, wps[2] = {wp2.x, wp2.y}, vps[2] = {vp2.x, vp2.y};
        float2 pf2[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float uf = ups[q] + wfj * (us[q] - ups[q]);
          const float wf = wps[q] + wfj * (ws[q] - wps[q]);
          pf2[q] = float2{(Uf + uf) * vps[q], (Wf + wf) * vps[q]};
        }
        F[sxi<float>(fslot * ngx + px)] = cat4(pf2[0], pf2[1]);
      }
    }
    __syncthreads();
    if (cprod || fprod) {
      float2* rows0[6];
      float2* rows1[6];
      int npair = 0;
      if (cprod) {
        for (int q = 0; q < 4; ++q) {
          rows0[q] = a.out[q] + (size_t)jj * d.mp + ro0;
          rows1[q] = a.out[q] + (size_t)jj * d.mp + ro1;
        }
        npair = 2;
      }
      if (fprod) {
        rows0[2 * npair] = a.out[4] + (size_t)(jj - 1) * d.mp + ro0;
        rows0[2 * npair + 1] = a.out[5] + (size_t)(jj - 1) * d.mp + ro0;
        rows1[2 * npair] = a.out[4] + (size_t)(jj - 1) * d.mp + ro1;
        rows1[2 * npair + 1] = a.out[5] + (size_t)(jj - 1) * d.mp + ro1;
        ++npair;
      }
      x_forward_pairs2(npair, F, rows0, rows1, d, pf);
    }
    float2* t;
    t = up; up = uc; uc = t;
    t = wp; wp = wc; wc = t;
    t = vp; vp = vc; vc = t;
  }
  if (a.want_cfl) {
    for (int o = 16; o > 0; o >>= 1) cmax = fmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
    if ((threadIdx.x & 31) == 0) cflred[threadIdx.x >> 5] = cmax;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, cflred[w]);
      atomicMax(&a.sc->cflbits, (unsigned long long)__double_as_longlong(m));
    }
  }
}

__global__ void __launch_bounds__(256) k_xprod2(const __grid_constant__ ProdArgs<float> a,
                                                const __grid_constant__ Dims d, const __grid_constant__ FftPlan ph,
                                                const __grid_constant__ FftPlan pf, const double2* __restrict__ rtw) {
  xprod2_body(a, d, ph, pf, rtw, blockIdx.x, blockIdx.y);
}

template <typename R>
void xprod_shape(const ProdArgs<R>& a, const Dims& d, dim3* grid, size_t* smem) {
  const int L0 = std::min(a.c_lo, a.f_lo + 1), L1 = std::max(a.c_hi, a.f_hi + 1);
  const int nlev = L1 - L0 + 1;
  if (sizeof(R) == 4 && a.rows == 2) {
    *grid = nlev <= 0 ? dim3(0, 0, 0) : dim3(d.ngz / 2, (nlev + a.chunk - 1) / a.chunk);
    *smem = sizeof(float4) * sx_elems<float>(3 * (size_t)d.ngx) + sizeof(float2) * 6 * (size_t)d.ngx;
    return;
  }
  *grid = nlev <= 0 ? dim3(0, 0, 0) : dim3(d.ngz, (nlev + a.chunk - 1) / a.chunk);
  *smem = sizeof(cpx_t<R>) * sx_elems<R>((a.split ? 2 : 3) * (size_t)d.ngx) + sizeof(R) * 6 * (size_t)d.ngx;
}

template <typename R>
void launch_xprod(const ProdArgs<R>& a, const Dims& d, const FftPlan& ph, const FftPlan& pf, const double2* rtw,
                  cudaStream_t st) {
  dim3 grid;
  size_t sm;
  xprod_shape(a, d, &grid, &sm);
  if (grid.x == 0) return;
  if constexpr (sizeof(R) == 4) {
    if (a.rows == 2) {
      k_xprod2<<<grid, a.threads == 128 ? 128 : 256, sm, st>>>(a, d, ph, pf, rtw);
      return;
    }
  }
  k_xprod<R><<<grid, a.threads == 128 ? 128 : 256, sm, st>>>(a, d, ph, pf, rtw);
}

// Canopy forcing on one mixed row of one processed plane: x-inverse, solid
// points set to 0 (or -beta*Luy on the tip planes), x-forward.
template <typename R>
__device__ __forceinline__ void xmask_body(const MaskArgs<R>& a, const Dims& d, const FftPlan& ph,
                                           const double2* __restrict__ rtw, int bx, int by) {
  using T2 = cpx_t<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ngx = d.ngx, h = ngx / 2, hp = h + 1;
  T2* F = reinterpret_cast<T2*>(smraw);
  R* rr = reinterpret_cast<R*>(F + sx_elems<R>(2 * (size_t)hp));
  R* ll = rr + ngx;
  const int kz = bx;
  int pl = by, f = 0;
  while (f < 2 && pl >= a.nplanes[f]) { pl -= a.nplanes[f]; ++f; }
  size_t plane = (size_t)by;
  T2* row = a.mix + plane * d.mp + (size_t)kz * d.nkx;
  const int tip = a.tipslot[f][pl];
  const uint8_t* msk = a.mask[f] + ((size_t)pl * d.ngz + kz) * ngx;
  // a row without solid points is unchanged by the forcing: its x round trip only drops the imaginary
  // part of its kx = 0 value (the real inverse ignores it), so that is all it needs
  int any = 0;
  for (int x = threadIdx.x; x < ngx; x += blockDim.x) any |= msk[x];
  if (!__syncthreads_or(any)) {
    if (threadIdx.x == 0) row[0].y = (R)0;
    return;
  }
  {
    const T2* rows[2] = {row, tip >= 0 ? a.lymix + (size_t)tip * d.mp + (size_t)kz * d.nkx : row};
    R* outs[2] = {rr, ll};
    x_inverse<R>(rows, tip >= 0 ? 2 : 1, F, hp, outs, d, ph, rtw);
  }
  const R mb = (R)(-a.beta);
  for (int m = threadIdx.x; m < h; m += blockDim.x) {
    R v[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int x = 2 * m + e;
      v[e] = rr[x];
      if (msk[x]) v[e] = (tip >= 0) ? mb * ll[x] : (R)0;
    }
    F[sxi<R>(ph.perm[m])] = T2{v[0], v[1]};
  }
  __syncthreads();
  T2* rows[1] = {row};
  x_forward_packed<R>(1, F, hp, rows, d, ph, rtw);
}

template <typename R>
__global__ void __launch_bounds__(128) k_xmask(const __grid_constant__ MaskArgs<R> a, const __grid_constant__ Dims d,
                                               const __grid_constant__ FftPlan ph, const double2* __restrict__ rtw) {
  xmask_body<R>(a, d, ph, rtw, blockIdx.x, blockIdx.y);
}

template <typename R>
void xmask_shape(const MaskArgs<R>& a, const Dims& d, dim3* grid, size_t* smem) {
  const int tot = a.nplanes[0] + a.nplanes[1] + a.nplanes[2];
  *grid = tot == 0 ? dim3(0, 0, 0) : dim3(d.ngz, tot);
  const int hp = d.ngx / 2 + 1;
  *smem = sizeof(cpx_t<R>) * sx_elems<R>(2 * (size_t)hp) + sizeof(R) * 2 * (size_t)d.ngx;
}

template <typename R>
void launch_xmask(const MaskArgs<R>& a, const Dims& d, const FftPlan& ph, const double2* rtw, cudaStream_t st) {
  dim3 grid;
  size_t sm;
  xmask_shape(a, d, &grid, &sm);
  if (grid.x == 0) return;
  k_xmask<R><<<grid, 128, sm, st>>>(a, d, ph, rtw);
}

// ---------------------------------------------------------------------------
// column-local kernels (always FP64)
// ---------------------------------------------------------------------------

__device__ __forceinline__ double2 ld(const double2* p) { return __ldg(p); }
__device__ __forceinline__ float2 ld(const float2* p) { return __ldg(p); }

// product spectra q = 0..5 (uu, uw, ww, vv, uv, vw) of the assembly's precision
template <typename P> __device__ __forceinline__ const P* prod(const AsmArgs& a, int q);
template <> __device__ __forceinline__ const double2* prod<double2>(const AsmArgs& a, int q) { return a.p64[q]; }
template <> __device__ __forceinline__ const float2* prod<float2>(const AsmArgs& a, int q) { return a.p32[q]; }

// The nonlinear term from the product spectra: (-kx A.y - kz B.y) + c (D1.x - D0.x) and its imaginary
// partner (d/dx, d/dz of the in-plane products, d/dy of the face products).  The mixed form's FP32
// spectra are combined in FP32 and only the result is widened.
__device__ __forceinline__ double2 nterm(double2 A, double2 B, double2 D1, double2 D0, double kx, double kz, double c) {
  return double2{(-kx * A.y - kz * B.y) + c * (D1.x - D0.x), (kx * A.x + kz * B.x) + c * (D1.y - D0.y)};
}
__device__ __forceinline__ double2 nterm(float2 A, float2 B, float2 D1, float2 D0, float fx, float fz, float fc) {
  return double2{(double)((-fx * A.y - fz * B.y) + fc * (D1.x - D0.x)),
                 (double)((fx * A.x + fz * B.x) + fc * (D1.y - D0.y))};
}
// the wavenumbers and the y metric in the precision the product spectra are combined in
template <typename P> __device__ __forceinline__ auto wnum(const double* d, const float* f, int i) {
  if constexpr (sizeof(P) == sizeof(float2)) return __ldg(f + i);
  else return d[i];
}

template <typename P>
__device__ __forceinline__ void assemble_body(const AsmArgs& a, const Dims& d, const Tables& t, int bx, int by) {
  const int col = bx * blockDim.x + threadIdx.x;
  if (col >= d.np) return;
  const int jj = by;
  const int np = d.np;
  const int i = col % d.nkx, kk = col / d.nkx;
  const double kx = t.kx[i], kz = t.kz[kk], k2 = t.k2x[i] + t.k2z[kk];
  // 1/axz of LUsolU/LUsolV (tridLU_3D_IB.f90:489,93) for this substage: a multiply instead of a
  // division, which costs ~10 FP64 instructions on a part with little FP64 throughput
  const double iaxz = t.iaxz[(size_t)a.k * np + col];
  const size_t c0 = (size_t)jj * np + col;
  const bool lng = is_long(d, i, kk);
  // u1 and u3 on centre jj
  const int lu = lev_u(d, lng, jj);
  if (lu != 1) {  // the column's end rows, or outside a short column
    a.r1[c0] = double2{0.0, 0.0};
    a.r3[c0] = double2{0.0, 0.0};
    if (lu == 0 || (jj != 0 && jj != d.nyu - 1)) {
      a.n1[c0] = double2{0.0, 0.0};
      a.n3[c0] = double2{0.0, 0.0};
    }
  } else {
    const double a1 = t.d2u[3 * jj], a2 = t.d2u[3 * jj + 1], a3 = t.d2u[3 * jj + 2];
    const double2 pc = ld(a.p + (size_t)(jj - 1) * np + col);
    const size_t f1 = (size_t)jj * np + col, f0 = f1 - np;  // faces jj and jj-1
    const bool tip = (jj == a.tipu[0] || jj == a.tipu[1]);
    const int tslot = (jj == a.tipu[0]) ? 0 : 1;
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const double2* u = f == 0 ? a.u1 : a.u3;
      const double2 um = ld(u + c0 - np), u0 = ld(u + c0), up = ld(u + c0 + np);
      const double L_x = a1 * um.x + (k2 + a2) * u0.x + a3 * up.x;
      const double L_y = a1 * um.y + (k2 + a2) * u0.y + a3 * up.y;
      const double kf = f == 0 ? kx : kz;
      // the first substage's zeta is 0 (start.f90:413-427): its old nonlinear term is not read, so a term left
      // from earlier fields (even a non-finite one) does not enter
      const double2 nold = a.C2 != 0.0 ? (f == 0 ? a.n1 : a.n3)[c0] : double2{0.0, 0.0};
      double rx = a.C1 * L_x + a.C2 * nold.x + (a.d * kf) * pc.y;
      double ry = a.C1 * L_y + a.C2 * nold.y + -(a.d * kf) * pc.x;
      if (f == 0 && col == 0) rx = rx + (-a.d * a.sc->mpgx);
      const P A = ld(prod<P>(a, f == 0 ? 0 : 1) + c0);
      const P B = ld(prod<P>(a, f == 0 ? 1 : 2) + c0);
      const P* D = prod<P>(a, f == 0 ? 4 : 5);
      // a short column's product is zero on the middle band's planes (they hold only long modes)
      const P D1 = (lng || !coarse_v(d, jj)) ? ld(D + f1) : P{0, 0};
      const P D0 = (lng || !coarse_v(d, jj - 1)) ? ld(D + f0) : P{0, 0};
      const double2 N = nterm(A, B, D1, D0, wnum<P>(t.kx, t.kxf, i), wnum<P>(t.kz, t.kzf, kk), wnum<P>(t.cu, t.cuf, jj));
      const double nr = N.x, ni = N.y;
      (f == 0 ? a.n1 : a.n3)[c0] = double2{nr, ni};
      rx = rx - a.g * nr;
      ry = ry - a.g * ni;
      (f == 0 ? a.r1 : a.r3)[c0] = double2{(u0.x + a.dt * rx) * iaxz, (u0.y + a.dt * ry) * iaxz};
      if (tip) {
        const double ly_x = a1 * um.x + (a2)*u0.x + a3 * up.x;
        const double ly_y = a1 * um.y + (a2)*u0.y + a3 * up.y;
        a.lytip[(size_t)(2 * f + tslot) * np + col] = double2{ly_x, ly_y};
      }
    }
  }
  // u2 on face jj
  if (jj <= d.nyv - 1) {
    const int lv = lev_v(d, lng, jj);
    if (lv != 1) {
      a.r2[c0] = double2{0.0, 0.0};
      if (lv == 0 || (jj != 0 && jj != d.nyv - 1)) a.n2[c0] = double2{0.0, 0.0};
    } else {
      const double a1 = t.d2v[3 * jj], a2 = t.d2v[3 * jj + 1], a3 = t.d2v[3 * jj + 2];
      const double2 um = ld(a.u2 + c0 - np), u0 = ld(a.u2 + c0), up = ld(a.u2 + c0 + np);
      const double2 p0 = ld(a.p + (size_t)(jj - 1) * np + col), p1 = ld(a.p + (size_t)jj * np + col);
      const double C3 = -a.d * t.cv[jj];
      const double L_x = a1 * um.x + (k2 + a2) * u0.x + a3 * up.x;
      const double L_y = a1 * um.y + (k2 + a2) * u0.y + a3 * up.y;
      const double2 nold = a.C2 != 0.0 ? a.n2[c0] : double2{0.0, 0.0};
      double rx = a.C1 * L_x + a.C2 * nold.x + C3 * (p1.x - p0.x);
      double ry = a.C1 * L_y + a.C2 * nold.y + C3 * (p1.y - p0.y);
      const P A = ld(prod<P>(a, 4) + c0), B = ld(prod<P>(a, 5) + c0);
      const P V1 = ld(prod<P>(a, 3) + c0 + np), V0 = ld(prod<P>(a, 3) + c0);
      const double2 N = nterm(A, B, V1, V0, wnum<P>(t.kx, t.kxf, i), wnum<P>(t.kz, t.kzf, kk), wnum<P>(t.cv, t.cvf, jj));
      const double nr = N.x, ni = N.y;
      a.n2[c0] = double2{nr, ni};
      rx = rx - a.g * nr;
      ry = ry - a.g * ni;
      a.r2[c0] = double2{(u0.x + a.dt * rx) * iaxz, (u0.y + a.dt * ry) * iaxz};
      if (jj == a.tipv[0] || jj == a.tipv[1]) {
        const int tslot = (jj == a.tipv[0]) ? 0 : 1;
        a.lytip[(size_t)(4 + tslot) * np + col] =
            double2{a1 * um.x + (a2)*u0.x + a3 * up.x, a1 * um.y + (a2)*u0.y + a3 * up.y};
      }
    }
  }
}

template <typename P>
__global__ void __launch_bounds__(256) k_assemble(const __grid_constant__ AsmArgs a, const __grid_constant__ Dims d,
                                                  const __grid_constant__ Tables t) {
  assemble_body<P>(a, d, t, blockIdx.x, blockIdx.y);
}

void launch_assemble(const AsmArgs& a, const Dims& d, const Tables& t, cudaStream_t st) {
  dim3 grid((d.np + 255) / 256, d.nyu);
  if (a.p32[0]) k_assemble<float2><<<grid, 256, 0, st>>>(a, d, t);
  else k_assemble<double2><<<grid, 256, 0, st>>>(a, d, t);
}

// Thomas sweeps of one column over levels lo..hi with an LU indexed by level
// (LUsolU/LUsolV, tridLU_3D_IB.f90:106-116,179-189); levels are prefetched
// four at a time.
__device__ __forceinline__ void thomas_column(double2* __restrict__ R, double2* __restrict__ U, size_t np, int col,
                                              const double* __restrict__ a1, const double* __restrict__ a2,
                                              const double* __restrict__ a3, int lo, int hi) {
  double2 x = R[(size_t)lo * np + col];
  x = double2{x.x * a2[lo], x.y * a2[lo]};
  R[(size_t)lo * np + col] = x;
  int jj = lo + 1;
  for (; jj + 3 <= hi; jj += 4) {
    double2 v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = R[(size_t)(jj + q) * np + col];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double b1 = a1[jj + q], b2 = a2[jj + q];
      x = double2{(v[q].x - b1 * x.x) * b2, (v[q].y - b1 * x.y) * b2};
      R[(size_t)(jj + q) * np + col] = x;
    }
  }
  for (; jj <= hi; ++jj) {
    const double2 v = R[(size_t)jj * np + col];
    x = double2{(v.x - a1[jj] * x.x) * a2[jj], (v.y - a1[jj] * x.y) * a2[jj]};
    R[(size_t)jj * np + col] = x;
  }
  U[(size_t)hi * np + col] = x;
  jj = hi - 1;
  for (; jj - 3 >= lo; jj -= 4) {
    double2 v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = R[(size_t)(jj - q) * np + col];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double b3 = a3[jj - q];
      x = double2{v[q].x - b3 * x.x, v[q].y - b3 * x.y};
      U[(size_t)(jj - q) * np + col] = x;
    }
  }
  for (; jj >= lo; --jj) {
    const double2 v = R[(size_t)jj * np + col];
    x = double2{v.x - a3[jj] * x.x, v.y - a3[jj] * x.y};
    U[(size_t)jj * np + col] = x;
  }
}

// Velocity solves: one thread per (component, column).  Long columns use the
// LU of the whole channel; short columns solve their two wall bands with those
// bands' LUs and are zero in between.
__device__ __forceinline__ void vsolve_body(double2* r1, double2* r2, double2* r3, double2* u1, double2* u2, double2* u3,
                                            const Dims& d, const Tables& t, int k, int bx, int by) {
  const int col = bx * blockDim.x + threadIdx.x;
  if (col >= d.np) return;
  const int comp = by;
  const int ny = comp == 1 ? d.nyv : d.nyu;
  double2* R = comp == 0 ? r1 : (comp == 1 ? r2 : r3);
  double2* U = comp == 0 ? u1 : (comp == 1 ? u2 : u3);
  const size_t np = d.np;
  const int i = col % d.nkx, kk = col / d.nkx;
  if (is_long(d, i, kk)) {
    const double* lu = comp == 1 ? t.lu_v + (size_t)k * 3 * d.nyv : t.lu_u + (size_t)k * 3 * d.nyu;
    thomas_column(R, U, np, col, lu, lu + ny, lu + 2 * ny, 0, ny - 1);
    return;
  }
  const double* l1 = (comp == 1 ? t.lu_v1 : t.lu_u1) + (size_t)k * 3 * ny;
  const double* l3 = (comp == 1 ? t.lu_v3 : t.lu_u3) + (size_t)k * 3 * ny;
  const int e1 = comp == 1 ? d.Nv1 + 1 : d.Nu1 + 1, s3 = comp == 1 ? d.Nv2 : d.Nu2;
  thomas_column(R, U, np, col, l1, l1 + ny, l1 + 2 * ny, 0, e1);
  thomas_column(R, U, np, col, l3, l3 + ny, l3 + 2 * ny, s3, ny - 1);
  for (int jj = e1 + 1; jj < s3; ++jj) U[(size_t)jj * np + col] = double2{0.0, 0.0};
}

__global__ void __launch_bounds__(128) k_vsolve(double2* r1, double2* r2, double2* r3, double2* u1, double2* u2,
                                                double2* u3, const __grid_constant__ Dims d,
                                                const __grid_constant__ Tables t, int k) {
  vsolve_body(r1, r2, r3, u1, u2, u3, d, t, k, blockIdx.x, blockIdx.y);
}

void launch_vsolve(double2* r1, double2* r2, double2* r3, double2* u1, double2* u2, double2* u3, const Dims& d,
                   const Tables& t, int k, cudaStream_t st) {
  dim3 grid((d.np + 127) / 128, 3);
  k_vsolve<<<grid, 128, 0, st>>>(r1, r2, r3, u1, u2, u3, d, t, k);
}

// flowrate_corr on mode (0,0): the flow-rate sum runs in the reference's
// order on one thread; the correction is spread over the block.
__device__ __forceinline__ void flowrate_body(double2* u1, DevScalars* sc, const Dims& d, const Tables& t, int k,
                                              double Qx1) {
  __shared__ double gsh;
  if (threadIdx.x == 0) {
    double Q = 0.0;
    for (int j = 1; j <= d.nn + 1; ++j) Q = Q + t.dyvw[j] * u1[(size_t)(j - d.ju0) * d.np].x;
    const double g = (sc->QxT - Q) / Qx1;
    sc->Qx = Q;
    sc->mpgx = sc->mpgx + g;
    gsh = g;
  }
  __syncthreads();
  const double g = gsh;
  const double* u11 = t.u11 + (size_t)k * (d.nn + 3);
  for (int j = threadIdx.x; j <= d.nn + 2; j += blockDim.x) {
    double2* u = u1 + (size_t)(j - d.ju0) * d.np;
    u->x = u->x + g * u11[j];
  }
}

__global__ void k_flowrate(double2* u1, DevScalars* sc, const __grid_constant__ Dims d, const __grid_constant__ Tables t,
                           int k, double Qx1) {
  flowrate_body(u1, sc, d, t, k, Qx1);
}

void launch_flowrate(double2* u1, DevScalars* sc, const Dims& d, const Tables& t, int k, double Qx1, cudaStream_t st) {
  k_flowrate<<<1, 256, 0, st>>>(u1, sc, d, t, k, Qx1);
}

// LU_buildP + LU_decP (tridLU_3D_IB.f90:497-571,643-684), one thread per
// column.  rows holds, per p level, the six products the matrix is made of:
// [0] D_b(j-1)*G_t(j)  [1] D_t(j)*G_b(j)  [2] D_b(j-1)*G_b(j-1)  [3] D_t(j)*G_t(j+1).
// LU_buildP + LU_decP (tridLU_3D_IB.f90:497-571,643-684) of one column over
// its p levels s0..e (rows: the column-independent D G products per level).
__device__ __forceinline__ void build_dg_segment(double* dg2, double* dg3, const double* rows, size_t np, int col,
                                                 double k2, bool dirichlet, double pin, int s0, int e) {
  double a2 = rows[4 * (size_t)s0 + 1] + k2;
  double a3 = rows[4 * (size_t)s0 + 3];
  if (dirichlet) { a2 = pin; a3 = 0.0; }
  a2 = 1.0 / a2;
  dg2[(size_t)s0 * np + col] = a2;
  for (int jp = s0 + 1; jp <= e; ++jp) {
    a3 = a3 * a2;                       // scaled upper diagonal of row jp-1
    dg3[(size_t)(jp - 1) * np + col] = a3;
    const double* q = rows + 4 * (size_t)jp;
    const double b2 = (jp < e) ? (q[0] + q[1]) + k2 : q[0] + k2;
    a2 = 1.0 / (b2 - q[2] * a3);
    dg2[(size_t)jp * np + col] = a2;
    a3 = (jp < e) ? q[3] : 0.0;
  }
  dg3[(size_t)e * np + col] = 0.0;
}

__global__ void k_build_dg(double* dg2, double* dg3, const double* rows, Dims d, Tables t, double pin) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= d.np) return;
  const int i = col % d.nkx, kk = col / d.nkx;
  const double k2 = t.k2x[i] + t.k2z[kk];
  const size_t np = d.np;
  if (is_long(d, i, kk)) {
    // mode (0,0): Dirichlet row for psi (tridLU_3D_IB.f90:548-554)
    build_dg_segment(dg2, dg3, rows, np, col, k2, col == 0, pin, 0, d.nyp - 1);
  } else {  // short column: its two wall bands, Neumann-like ends at the band edges
    build_dg_segment(dg2, dg3, rows, np, col, k2, false, pin, 0, d.Nu1 - 1);
    build_dg_segment(dg2, dg3, rows, np, col, k2, false, pin, d.Nu2, d.nyp - 1);
  }
}

void launch_build_dg(double* dg2, double* dg3, const double* rows, const Dims& d, const Tables& t, double pin,
                     cudaStream_t st) {
  k_build_dg<<<(d.np + 127) / 128, 128, 0, st>>>(dg2, dg3, rows, d, t, pin);
}

// solveP + v_corr over the p levels lo..hi of one column (a long column's all,
// or one wall band of a short one).  The divergence is formed on the fly in
// the forward sweep; the backward sweep adds psi to p and corrects u, w on the
// same levels and v on the faces between them.
// bit pattern test for a NaN or an infinity (integer work only, off the FP64 pipe)
__device__ __forceinline__ bool nonfinite(double x) {
  return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
}

__device__ __forceinline__ void psolve_segment(double2* __restrict__ u1, double2* __restrict__ u2,
                                               double2* __restrict__ u3, double2* __restrict__ p,
                                               double2* __restrict__ psi, const Dims& d, const Tables& t, int col,
                                               double kx, double kz, double dtirk, double dtrk, int lo, int hi,
                                               bool pin00, bool& bad) {
  // levels are loaded four at a time ahead of the recurrences (the arithmetic and its order are those of
  // one level at a time)
  const size_t np = d.np;
  const double* __restrict__ dg2 = t.dg2;
  const double* __restrict__ dg3 = t.dg3;
  double2 x = double2{0.0, 0.0};
  double2 vlo = u2[(size_t)lo * np + col];  // v on face jp, carried from the level below
  auto fwd = [&](int jp, const double2& a, const double2& w, const double2& v1, const double2& v0, double b2) {
    const double c = t.cu[jp + 1];
    const double2 dv = double2{(-kx * a.y - kz * w.y) + c * (v1.x - v0.x), (kx * a.x + kz * w.x) + c * (v1.y - v0.y)};
    double2 ps = double2{dtirk * dv.x, dtirk * dv.y};
    if (pin00 && jp == lo) ps = double2{0.0, 0.0};
    if (jp == lo) x = double2{ps.x * b2, ps.y * b2};
    else {
      const double b1 = t.dg1[jp];
      x = double2{(ps.x - b1 * x.x) * b2, (ps.y - b1 * x.y) * b2};
    }
    psi[(size_t)jp * np + col] = x;
  };
  int jp = lo;
  for (; jp + 3 <= hi; jp += 4) {
    double2 A[4], W[4], V[4];
    double B2[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const size_t cu = (size_t)(jp + q + 1) * np + col;
      A[q] = u1[cu];
      W[q] = u3[cu];
      V[q] = u2[cu];
      B2[q] = dg2[(size_t)(jp + q) * np + col];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) fwd(jp + q, A[q], W[q], V[q], q == 0 ? vlo : V[q - 1], B2[q]);
    vlo = V[3];
  }
  for (; jp <= hi; ++jp) {
    const size_t cu = (size_t)(jp + 1) * np + col;
    const double2 v1 = u2[cu];
    fwd(jp, u1[cu], u3[cu], v1, vlo, dg2[(size_t)jp * np + col]);
    vlo = v1;
  }
  const double kxd = dtrk * kx, kzd = dtrk * kz;
  double2 xn = x;  // psi(hi)
  auto bwd = [&](int jq, const double2& v, double b3, const double2& pp, const double2& a, const double2& w,
                 const double2& vv) {
    const double2 xc = jq == hi ? xn : double2{v.x - b3 * xn.x, v.y - b3 * xn.y};
    const size_t cp = (size_t)jq * np + col, cu = (size_t)(jq + 1) * np + col;
    const double2 pn = double2{pp.x + xc.x, pp.y + xc.y};
    // a NaN or infinity anywhere in the fields reaches the divergence of its column, hence psi and p
    bad = bad || nonfinite(pn.x) || nonfinite(pn.y);
    p[cp] = pn;
    u1[cu] = double2{a.x - (-kxd * xc.y), a.y - (kxd * xc.x)};
    u3[cu] = double2{w.x - (-kzd * xc.y), w.y - (kzd * xc.x)};
    if (jq < hi) {
      const double f = dtrk * t.cv[jq + 1];
      u2[cu] = double2{vv.x - f * (xn.x - xc.x), vv.y - f * (xn.y - xc.y)};
    }
    xn = xc;
  };
  jp = hi;
  for (; jp - 3 >= lo; jp -= 4) {
    double2 Ps[4], P[4], A[4], W[4], V[4];
    double B3[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int jq = jp - q;
      const size_t cp = (size_t)jq * np + col, cu = (size_t)(jq + 1) * np + col;
      Ps[q] = psi[cp];
      B3[q] = dg3[cp];
      P[q] = p[cp];
      A[q] = u1[cu];
      W[q] = u3[cu];
      V[q] = u2[cu];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) bwd(jp - q, Ps[q], B3[q], P[q], A[q], W[q], V[q]);
  }
  for (; jp >= lo; --jp) {
    const size_t cp = (size_t)jp * np + col, cu = (size_t)(jp + 1) * np + col;
    bwd(jp, psi[cp], dg3[cp], p[cp], u1[cu], u3[cu], u2[cu]);
  }
}

__device__ __forceinline__ void psolve_body(double2* u1, double2* u2, double2* u3, double2* p, double2* psi, const Dims& d,
                                            const Tables& t, double dtirk, double dtrk, double gwb, double gwt,
                                            DevScalars* sc, int bx) {
  const int col = bx * blockDim.x + threadIdx.x;
  if (col >= d.np) return;
  const size_t np = d.np;
  const int i = col % d.nkx, kk = col / d.nkx;
  const double kx = t.kx[i], kz = t.kz[kk];
  bool bad = false;
  if (is_long(d, i, kk)) {
    psolve_segment(u1, u2, u3, p, psi, d, t, col, kx, kz, dtirk, dtrk, 0, d.nyp - 1, col == 0, bad);
  } else {
    psolve_segment(u1, u2, u3, p, psi, d, t, col, kx, kz, dtirk, dtrk, 0, d.Nu1 - 1, false, bad);
    psolve_segment(u1, u2, u3, p, psi, d, t, col, kx, kz, dtirk, dtrk, d.Nu2, d.nyp - 1, false, bad);
    // v on the end rows of the short column's bands (v_corr, littleharsh.f90:904-905)
    u2[(size_t)(d.Nv1 + 1) * np + col] = double2{0.0, 0.0};
    u2[(size_t)d.Nv2 * np + col] = double2{0.0, 0.0};
  }
  u2[col] = double2{0.0, 0.0};
  u2[(size_t)(d.nyv - 1) * np + col] = double2{0.0, 0.0};
  {
    const double2 a = u1[np + col], w = u3[np + col];
    u1[col] = double2{-gwb * a.x, -gwb * a.y};
    u3[col] = double2{-gwb * w.x, -gwb * w.y};
    const double2 at = u1[(size_t)(d.nyu - 2) * np + col], wt = u3[(size_t)(d.nyu - 2) * np + col];
    u1[(size_t)(d.nyu - 1) * np + col] = double2{-gwt * at.x, -gwt * at.y};
    u3[(size_t)(d.nyu - 1) * np + col] = double2{-gwt * wt.x, -gwt * wt.y};
  }
  if (bad && sc) atomicOr(&sc->err, kErrNonFinite);
}

__global__ void __launch_bounds__(128, 4) k_psolve(double2* u1, double2* u2, double2* u3, double2* p, double2* psi,
                                                   const __grid_constant__ Dims d, const __grid_constant__ Tables t,
                                                   double dtirk, double dtrk, double gwb, double gwt, DevScalars* sc) {
  psolve_body(u1, u2, u3, p, psi, d, t, dtirk, dtrk, gwb, gwt, sc, blockIdx.x);
}

void launch_psolve(double2* u1, double2* u2, double2* u3, double2* p, double2* psi, const Dims& d, const Tables& t,
                   double dtirk, double dtrk, double gwb, double gwt, DevScalars* sc, cudaStream_t st) {
  dim3 grid((d.np + 127) / 128);
  k_psolve<<<grid, 128, 0, st>>>(u1, u2, u3, p, psi, d, t, dtirk, dtrk, gwb, gwt, sc);
}

__global__ void k_divergence(const double2* u1, const double2* u2, const double2* u3, double2* div, Dims d, Tables t) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= d.np) return;
  const int jp = blockIdx.y, ju = jp + 1;
  const size_t np = d.np;
  const int i = col % d.nkx, kk = col / d.nkx;
  if (!lev_p(d, is_long(d, i, kk), jp)) { div[(size_t)jp * np + col] = double2{0.0, 0.0}; return; }
  const double kx = t.kx[i], kz = t.kz[kk];
  const double2 a = u1[(size_t)ju * np + col], w = u3[(size_t)ju * np + col];
  const double2 v1 = u2[(size_t)ju * np + col], v0 = u2[(size_t)jp * np + col];
  const double c = t.cu[ju];
  div[(size_t)jp * np + col] =
      double2{(-kx * a.y - kz * w.y) + c * (v1.x - v0.x), (kx * a.x + kz * w.x) + c * (v1.y - v0.y)};
}

void launch_divergence(const double2* u1, const double2* u2, const double2* u3, double2* div, const Dims& d,
                       const Tables& t, cudaStream_t st) {
  dim3 grid((d.np + 255) / 256, d.nyp);
  k_divergence<<<grid, 256, 0, st>>>(u1, u2, u3, div, d, t);
}

__global__ void k_absmax(const double2* x, size_t n, DevScalars* sc) {
  double m = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    m = fmax(m, hypot(x[e].x, x[e].y));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&sc->cflbits, (unsigned long long)__double_as_longlong(m));
}

void launch_absmax(const double2* x, size_t n, DevScalars* sc, cudaStream_t st) {
  k_absmax<<<152 * 4, 256, 0, st>>>(x, n, sc);
}

// [rows][cols] -> [cols][rows] through a shared-memory tile.
__global__ void k_gather_col(const double2* __restrict__ src, size_t stride, int n, double2* __restrict__ dst) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) dst[j] = src[(size_t)j * stride];
}

void launch_gather_col(const double2* src, size_t stride, int n, double2* dst, cudaStream_t st) {
  if (n > 0) k_gather_col<<<(n + 127) / 128, 128, 0, st>>>(src, stride, n, dst);
}

__global__ void k_transpose(const double2* __restrict__ src, double2* __restrict__ dst, int rows, int cols) {
  __shared__ double2 tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int row = by + r, c = bx + threadIdx.x;
    if (row < rows && c < cols) tile[r][threadIdx.x] = src[(size_t)row * cols + c];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int c = bx + r, row = by + threadIdx.x;
    if (row < rows && c < cols) dst[(size_t)c * rows + row] = tile[threadIdx.x][r];
  }
}

void launch_transpose(const double2* src, double2* dst, int rows, int cols, cudaStream_t st) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  k_transpose<<<grid, dim3(32, 8), 0, st>>>(src, dst, rows, cols);
}

// spectra.f90:18-56: sums of |u|^2, |v|^2, |w|^2, Re(u conj v_c), |p|^2 per (level, column).
// sp layout: [spU nyu][spV nyv][spW nyu][spUV nyu][spP nyp] planes of np doubles.
__global__ void k_spectra(const double2* u1, const double2* u2, const double2* u3, const double2* p, double* sp,
                          Dims d, Tables t) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= d.np) return;
  const int jj = blockIdx.y;
  const size_t np = d.np;
  double* spU = sp;
  double* spV = spU + (size_t)d.nyu * np;
  double* spW = spV + (size_t)d.nyv * np;
  double* spUV = spW + (size_t)d.nyu * np;
  double* spP = spUV + (size_t)d.nyu * np;
  const size_t c0 = (size_t)jj * np + col;
  if (jj < d.nyu) {
    const double2 a = u1[c0], w = u3[c0];
    spU[c0] = spU[c0] + a.x * a.x + a.y * a.y;
    spW[c0] = spW[c0] + w.x * w.x + w.y * w.y;
    double2 vi = double2{0.0, 0.0};
    if (jj >= 1 && jj <= d.nyu - 2) {
      const double2 v0 = u2[c0 - np], v1 = u2[c0];
      const double wc = t.wc[jj];
      vi = double2{v0.x + wc * (v1.x - v0.x), v0.y + wc * (v1.y - v0.y)};
    }
    spUV[c0] = spUV[c0] + a.x * vi.x + a.y * vi.y;
  }
  if (jj < d.nyv) {
    const double2 v = u2[c0];
    spV[c0] = spV[c0] + v.x * v.x + v.y * v.y;
  }
  if (jj < d.nyp) {
    const double2 q = p[c0];
    spP[c0] = spP[c0] + q.x * q.x + q.y * q.y;
  }
}

// Plane statistics of stats.f90:1-108 (sums over the physical plane of each
// level), accumulated without transforms: the physical plane is the exact
// inverse DFT of the zero-padded spectrum, so by Parseval
//   sum_{x,z} f g = Ngx Ngz [ sum_{kx>0} 2 Re(f g*) + sum_kz h_f h_g* ],
// where h is the kx = 0 line made Hermitian the way the real x-inverse
// makes it (its imaginary part is dropped; the lone kz = -N2/2 mode splits
// into -N2/2 and +N2/2 on the padded grid).  sum f = Ngx Ngz Re f(0,0).
// acc rows (length L = max(nyu, nyv)): 0 Um 1 U2m 2 Vm 3 V2m 4 Wm 5 W2m 6 Pm 7 P2m
// 8 UVm (u, v at centres) 9 UWm 10 VWm (v, w at faces) 11 wxm 12 wx2m (omega_x
// at faces, omega_at_face below).  One block per level.
// With bands a plane of the middle band sums over its own points: only the long
// columns count, the lone mode is that band's -N2/2 and the factor its Ngx Ngz.
__device__ __forceinline__ double pair_term(const double2* f, const double2* g, int col, int i, int kk, int nz,
                                            int nkx, int lone) {
  const double2 a = f[col], b = g[col];
  const double re = a.x * b.x + a.y * b.y;  // Re(a conj b)
  if (i > 0) return 2.0 * re;
  if (kk == lone) return 0.5 * re;
  const int pk = (nz - kk) % nz;
  const double2 c = g[(size_t)pk * nkx];
  return 0.5 * (re + (a.x * c.x - a.y * c.y));  // + Re(a g(-kz))
}

// Streamwise vorticity omega_x = dw/dy - dv/dz at face jj of column col (the wx
// planes of stats.f90:53-58,93,102, filled in the reference by the missing
// FOU3D.f90): the y-difference of w across the face with the pressure
// gradient's metric (littleharsh.f90:685) minus i kz v.
__device__ __forceinline__ double2 omega_at_face(const double2* u2, const double2* u3, const Dims& d, const Tables& t,
                                                 int jj, int col) {
  const size_t np = d.np;
  const double c = t.cv[jj], kz = t.kz[col / d.nkx];
  const double2 w0 = u3[(size_t)jj * np + col], w1 = u3[(size_t)(jj + 1) * np + col], v = u2[(size_t)jj * np + col];
  return double2{c * (w1.x - w0.x) + kz * v.y, c * (w1.y - w0.y) - kz * v.x};
}

__global__ void __launch_bounds__(256) k_stats(const double2* u1, const double2* u2, const double2* u3,
                                               const double2* p, double2* vc, double2* wf, double2* om, double* acc,
                                               Dims d, Tables t, int L) {
  const int jj = blockIdx.x;
  const size_t np = d.np;
  double s[13];
#pragma unroll
  for (int r = 0; r < 13; ++r) s[r] = 0.0;
  // v at the centre jj, w at the face jj (zero on ghost centres and wall faces) and omega_x at the face jj
  double2* vcl = vc + (size_t)blockIdx.x * np;
  double2* wfl = wf + (size_t)blockIdx.x * np;
  double2* oml = om + (size_t)blockIdx.x * np;
  const bool cin = jj >= 1 && jj <= d.nyu - 2, fin = jj >= 1 && jj <= d.nyv - 2;
  for (int col = threadIdx.x; col < d.np; col += blockDim.x) {
    if (jj < d.nyv) oml[col] = omega_at_face(u2, u3, d, t, jj, col);
    double2 v = double2{0.0, 0.0}, w = double2{0.0, 0.0};
    if (cin) {
      const double2 v0 = u2[(size_t)(jj - 1) * np + col], v1 = u2[(size_t)jj * np + col];
      const double c = t.wc[jj];
      v = double2{v0.x + c * (v1.x - v0.x), v0.y + c * (v1.y - v0.y)};
    }
    if (fin) {
      const double2 w0 = u3[(size_t)jj * np + col], w1 = u3[(size_t)(jj + 1) * np + col];
      const double c = t.wf[jj];
      w = double2{w0.x + c * (w1.x - w0.x), w0.y + c * (w1.y - w0.y)};
    }
    vcl[col] = v;
    wfl[col] = w;
  }
  __syncthreads();
  const double2* U = u1 + (size_t)jj * np;
  const double2* W = u3 + (size_t)jj * np;
  const double2* V = u2 + (size_t)jj * np;
  const double2* P = p + (size_t)jj * np;
  // plane of each group: u quantities at centre jj, v ones at face jj, p at p level jj (centre jj + 1)
  const bool cu_ = coarse_u(d, jj), cv_ = coarse_v(d, jj), cp_ = coarse_u(d, jj + 1);
  const int lone_f = d.nz / 2, lone_c = d.nz - d.nz2 / 2;
  for (int col = threadIdx.x; col < d.np; col += blockDim.x) {
    const int i = col % d.nkx, kk = col / d.nkx;
    const bool lng = is_long(d, i, kk);
    if (jj < d.nyu && (lng || !cu_)) {
      const int lone = cu_ ? lone_c : lone_f;
      s[1] += pair_term(U, U, col, i, kk, d.nz, d.nkx, lone);
      s[5] += pair_term(W, W, col, i, kk, d.nz, d.nkx, lone);
      s[8] += pair_term(U, vcl, col, i, kk, d.nz, d.nkx, lone);
      s[9] += pair_term(U, W, col, i, kk, d.nz, d.nkx, lone);
    }
    if (jj < d.nyv && (lng || !cv_)) {
      const int lone = cv_ ? lone_c : lone_f;
      s[3] += pair_term(V, V, col, i, kk, d.nz, d.nkx, lone);
      s[10] += pair_term(V, wfl, col, i, kk, d.nz, d.nkx, lone);
      s[12] += pair_term(oml, oml, col, i, kk, d.nz, d.nkx, lone);
    }
    if (jj < d.nyp && (lng || !cp_)) s[7] += pair_term(P, P, col, i, kk, d.nz, d.nkx, cp_ ? lone_c : lone_f);
  }
  if (threadIdx.x == 0) {
    if (jj < d.nyu) { s[0] = U[0].x; s[4] = W[0].x; }
    if (jj < d.nyv) { s[2] = V[0].x; s[11] = oml[0].x; }
    if (jj < d.nyp) s[6] = P[0].x;
  }
  __shared__ double red[8][13];
#pragma unroll
  for (int r = 0; r < 13; ++r) {
    double x = s[r];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][r] = x;
  }
  __syncthreads();
  if (threadIdx.x < 13) {
    double x = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x += red[w][threadIdx.x];
    const int r = threadIdx.x;
    const bool coarse = (r == 2 || r == 3 || r >= 10) ? cv_ : ((r == 6 || r == 7) ? cp_ : cu_);
    const double scale = coarse ? (double)d.ngx2 * (double)d.ngz2 : (double)d.ngx * (double)d.ngz;
    acc[(size_t)r * L + jj] += scale * x;
  }
}

void launch_stats(const double2* u1, const double2* u2, const double2* u3, const double2* p, double2* vc,
                  double2* wf, double2* om, double* acc, const Dims& d, const Tables& t, cudaStream_t st) {
  const int L = d.nyu > d.nyv ? d.nyu : d.nyv;
  k_stats<<<L, 256, 0, st>>>(u1, u2, u3, p, vc, wf, om, acc, d, t, L);
}

// v interpolated to every centre and w to every face in spectral space (zero
// on ghost centres and wall faces): the y interpolation the statistics pair
// u with v and v with w through.
__global__ void k_stage_itp(const double2* u2, const double2* u3, double2* vc, double2* wf, double2* om, Dims d,
                            Tables t) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= d.np) return;
  const int jj = blockIdx.y;
  const size_t np = d.np, c0 = (size_t)jj * np + col;
  if (jj < d.nyu) {
    double2 v = double2{0.0, 0.0};
    if (jj >= 1 && jj <= d.nyu - 2) {
      const double2 v0 = u2[c0 - np], v1 = u2[c0];
      const double c = t.wc[jj];
      v = double2{v0.x + c * (v1.x - v0.x), v0.y + c * (v1.y - v0.y)};
    }
    vc[c0] = v;
  }
  if (jj < d.nyv) {
    double2 w = double2{0.0, 0.0};
    if (jj >= 1 && jj <= d.nyv - 2) {
      const double2 w0 = u3[c0], w1 = u3[c0 + np];
      const double c = t.wf[jj];
      w = double2{w0.x + c * (w1.x - w0.x), w0.y + c * (w1.y - w0.y)};
    }
    wf[c0] = w;
    if (om) om[c0] = omega_at_face(u2, u3, d, t, jj, col);
  }
}

void launch_stage_itp(const double2* u2, const double2* u3, double2* vc, double2* wf, double2* om, const Dims& d,
                      const Tables& t, cudaStream_t st) {
  dim3 grid((d.np + 255) / 256, d.nyu);
  k_stage_itp<<<grid, 256, 0, st>>>(u2, u3, vc, wf, om, d, t);
}

// Conditional statistics (conddown1/2, condup1/2: stats.f90:110-253; both
// walls summed as recvXC does, stats.f90:473-512).  One CTA per (grid g,
// plane j1 of this chunk, in-tile z index kin): for each of the ntilez rows
// of that z phase and each wall it x-inverts the mixed rows and adds the row
// folded onto the dnx in-tile x points.  Plane 2*jl + side of the mixed
// buffers holds wall `side` (0 bottom, 1 top mirrored) of plane j1 = j0 + jl.
__global__ void __launch_bounds__(128) k_xcond(CondArgs a, Dims d, FftPlan ph, const double2* __restrict__ rtw) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ngx = d.ngx, h = ngx / 2, hp = h + 1;
  double2* F = reinterpret_cast<double2*>(smraw);
  double* rows = reinterpret_cast<double*>(F + 3 * hp);
  double* acc = rows + 3 * ngx;  // [6][dnx]
  const int g = blockIdx.z, jl = blockIdx.x, kin = blockIdx.y;
  const int nj = a.nj[g];
  if (jl >= nj) return;
  const int nf = g == 2 ? 1 : 3;
  const int nq = g == 0 ? 6 : (g == 1 ? 5 : 2);
  for (int e = threadIdx.x; e < 6 * a.dnx; e += blockDim.x) acc[e] = 0.0;
  __syncthreads();
  for (int iz = 0; iz < a.ntz; ++iz) {
    const size_t rowoff = (size_t)(kin + a.dnz * iz) * d.nkx;
    for (int side = 0; side < 2; ++side) {
      const size_t plane = (size_t)(2 * jl + side) * d.mp;
      const double2* src[3];
      double* outs[3] = {rows, rows + ngx, rows + 2 * ngx};
      for (int f = 0; f < nf; ++f) src[f] = a.mix[g][f] + plane + rowoff;
      x_inverse<double>(src, nf, F, hp, outs, d, ph, rtw);
      const double sg = side ? -1.0 : 1.0;
      for (int i = threadIdx.x; i < a.dnx; i += blockDim.x) {
        double q[6] = {0, 0, 0, 0, 0, 0};
        for (int ix = 0; ix < a.ntx; ++ix) {
          const int x = i + a.dnx * ix;
          const double A = rows[x];
          if (g == 0) {
            const double B = rows[ngx + x], C = rows[2 * ngx + x];
            q[0] += A; q[1] += A * A; q[2] += B; q[3] += B * B; q[4] += A * (sg * C); q[5] += A * B;
          } else if (g == 1) {
            // omega_x keeps its sign on the top wall (condup1 called with xsign = 1 for wx, stats.f90:102)
            const double B = rows[ngx + x], C = rows[2 * ngx + x];
            q[0] += sg * A; q[1] += A * A; q[2] += (sg * A) * B; q[3] += C; q[4] += C * C;
          } else {
            q[0] += A; q[1] += A * A;
          }
        }
        for (int r = 0; r < nq; ++r) acc[r * a.dnx + i] += q[r];
      }
      __syncthreads();
    }
  }
  const size_t pl = (size_t)a.dnx * a.dnz;
  for (int i = threadIdx.x; i < a.dnx; i += blockDim.x)
    for (int r = 0; r < nq; ++r) {
      // the v grid's omega_x sums (quantities 3, 4) have their own blocks after the p grid's
      double* base = (g == 1 && r >= 3) ? a.outw + (size_t)(r - 3) * a.njtot[1] * pl
                                        : a.out[g] + (size_t)r * a.njtot[g] * pl;
      double* o = base + (size_t)(a.j0 + jl) * pl + (size_t)kin * a.dnx + i;
      *o += acc[r * a.dnx + i];
    }
}

void launch_xcond(const CondArgs& a, const Dims& d, const FftPlan& ph, const double2* rtw, cudaStream_t st) {
  const int njmax = a.nj[0] > a.nj[1] ? (a.nj[0] > a.nj[2] ? a.nj[0] : a.nj[2]) : (a.nj[1] > a.nj[2] ? a.nj[1] : a.nj[2]);
  if (njmax <= 0) return;
  dim3 grid(njmax, a.dnz, 3);
  const int hp = d.ngx / 2 + 1;
  size_t sm = sizeof(double2) * 3 * (size_t)hp + sizeof(double) * (3 * (size_t)d.ngx + 6 * (size_t)a.dnx);
  k_xcond<<<grid, 128, sm, st>>>(a, d, ph, rtw);
}

void launch_spectra(const double2* u1, const double2* u2, const double2* u3, const double2* p, double* sp,
                    const Dims& d, const Tables& t, cudaStream_t st) {
  dim3 grid((d.np + 255) / 256, d.nyu);
  k_spectra<<<grid, 256, 0, st>>>(u1, u2, u3, p, sp, d, t);
}

// ---------------------------------------------------------------------------
// Batched kernels (several solvers per launch, lh_internal.h)
// ---------------------------------------------------------------------------

// The batched kernels read their member's arguments with a block-uniform index into the parameter bank, which
// costs registers the single launches do not need; their launch bounds cap the registers at the single
// launches' counts, so that as many CTAs fit on an SM.

// member owning block b (members are few; the scan is uniform across the block)
template <typename D>
__device__ __forceinline__ int batch_member(const Batch<D>& b, int blk) {
  int m = 0;
  while (m + 1 < b.n && blk >= b.start[m + 1]) ++m;
  return m;
}

template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 8 : 5) k_zinv_batch(const __grid_constant__ Batch<ZDesc<R>> b) {
  const int m = batch_member(b, blockIdx.x);
  const ZDesc<R>& D = b.desc[m];
  const int q = blockIdx.x - b.start[m], gxy = D.gx * D.gy;
  zinv_body<R>(D.jobs, D.d, D.p, D.tx, q % D.gx, (q % gxy) / D.gx, q / gxy);
}

template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 8 : 5) k_zfwd_batch(const __grid_constant__ Batch<ZDesc<R>> b) {
  const int m = batch_member(b, blockIdx.x);
  const ZDesc<R>& D = b.desc[m];
  const int q = blockIdx.x - b.start[m], gxy = D.gx * D.gy;
  zfwd_body<R>(D.jobs, D.d, D.p, D.tx, D.scale, q % D.gx, (q % gxy) / D.gx, q / gxy);
}

template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 6 : 5) k_xprod_batch(const __grid_constant__ Batch<XDesc<R>> b) {
  const int m = batch_member(b, blockIdx.x);
  const XDesc<R>& D = b.desc[m];
  const int q = blockIdx.x - b.start[m];
  xprod_body<R>(D.a, D.d, D.ph, D.pf, D.rtw, q % D.gx, q / D.gx);
}

template <typename R>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 16 : 9) k_xmask_batch(const __grid_constant__ Batch<MDesc<R>> b) {
  const int m = batch_member(b, blockIdx.x);
  const MDesc<R>& D = b.desc[m];
  const int q = blockIdx.x - b.start[m];
  xmask_body<R>(D.a, D.d, D.ph, D.rtw, q % D.gx, q / D.gx);
}

template <typename P>
__global__ void __launch_bounds__(256, 3) k_assemble_batch(const __grid_constant__ Batch<ADesc> b) {
  const int m = batch_member(b, blockIdx.x);
  const ADesc& D = b.desc[m];
  const int q = blockIdx.x - b.start[m];
  assemble_body<P>(D.a, D.d, D.t, q % D.gx, q / D.gx);
}

__global__ void __launch_bounds__(128) k_vsolve_batch(const __grid_constant__ Batch<VDesc> b) {
  const int m = batch_member(b, blockIdx.x);
  const VDesc& D = b.desc[m];
  const int q = blockIdx.x - b.start[m];
  vsolve_body(D.r1, D.r2, D.r3, D.u1, D.u2, D.u3, D.d, D.t, D.k, q % D.gx, q / D.gx);
}

__global__ void k_flowrate_batch(const __grid_constant__ Batch<FDesc> b) {
  const FDesc& D = b.desc[batch_member(b, blockIdx.x)];
  flowrate_body(D.u1, D.sc, D.d, D.t, D.k, D.Qx1);
}

__global__ void __launch_bounds__(128, 4) k_psolve_batch(const __grid_constant__ Batch<PDesc> b) {
  const int m = batch_member(b, blockIdx.x);
  const PDesc& D = b.desc[m];
  psolve_body(D.u1, D.u2, D.u3, D.p, D.psi, D.d, D.t, D.dtirk, D.dtrk, D.gwb, D.gwt, D.sc, blockIdx.x - b.start[m]);
}

template <typename R>
void launch_zinv_batch(const Batch<ZDesc<R>>& b, size_t smem, cudaStream_t st) {
  if (b.n > 0 && b.start[b.n] > 0) k_zinv_batch<R><<<b.start[b.n], 256, smem, st>>>(b);
}
template <typename R>
void launch_zfwd_batch(const Batch<ZDesc<R>>& b, size_t smem, cudaStream_t st) {
  if (b.n > 0 && b.start[b.n] > 0) k_zfwd_batch<R><<<b.start[b.n], 256, smem, st>>>(b);
}
template <typename R>
void launch_xprod_batch(const Batch<XDesc<R>>& b, size_t smem, cudaStream_t st) {
  if (b.n > 0 && b.start[b.n] > 0) k_xprod_batch<R><<<b.start[b.n], 256, smem, st>>>(b);
}
template <typename R>
void launch_xmask_batch(const Batch<MDesc<R>>& b, size_t smem, cudaStream_t st) {
  if (b.n > 0 && b.start[b.n] > 0) k_xmask_batch<R><<<b.start[b.n], 128, smem, st>>>(b);
}
void launch_assemble_batch(const Batch<ADesc>& b, bool fp32_products, cudaStream_t st) {
  if (b.n <= 0 || b.start[b.n] <= 0) return;
  if (fp32_products) k_assemble_batch<float2><<<b.start[b.n], 256, 0, st>>>(b);
  else k_assemble_batch<double2><<<b.start[b.n], 256, 0, st>>>(b);
}
void launch_vsolve_batch(const Batch<VDesc>& b, cudaStream_t st) {
  if (b.n > 0 && b.start[b.n] > 0) k_vsolve_batch<<<b.start[b.n], 128, 0, st>>>(b);
}
void launch_flowrate_batch(const Batch<FDesc>& b, cudaStream_t st) {
  if (b.n > 0 && b.start[b.n] > 0) k_flowrate_batch<<<b.start[b.n], 256, 0, st>>>(b);
}
void launch_psolve_batch(const Batch<PDesc>& b, cudaStream_t st) {
  if (b.n > 0 && b.start[b.n] > 0) k_psolve_batch<<<b.start[b.n], 128, 0, st>>>(b);
}

// FP64 FMA throughput probe: every thread runs eight independent dependent
// chains of fma(x, a, b), enough independent work to keep the FP64 pipe busy;
// the sum is stored only if it equals an impossible value, so no chain is
// removed by the compiler.
__global__ void __launch_bounds__(256) k_fp64_probe(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) x[q] = 1e-9 * threadIdx.x + q;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = fma(x[q], a, b);
  }
  double sum = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) sum += x[q];
  if (sum == -1.0) out[blockIdx.x] = sum;
}

double fp64_probe_tflops(int* nsm_out) {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return -1.0;
  if (nsm_out) *nsm_out = nsm;
  const int blocks = nsm * 8, threads = 256, iters = 4096;
  double* out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double best = -1.0;
  if (cudaMalloc(&out, sizeof(double) * blocks) == cudaSuccess && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
      cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
    k_fp64_probe<<<blocks, threads, 0, st>>>(out, iters / 8, 0.9999999, 1e-7);  // warm-up
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, st);
      k_fp64_probe<<<blocks, threads, 0, st>>>(out, iters, 0.9999999, 1e-7);
      cudaEventRecord(e1, st);
      if (cudaEventSynchronize(e1) != cudaSuccess) { best = -1.0; break; }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
      const double tf = flops / (ms * 1e-3) / 1e12;
      if (tf > best) best = tf;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  return best;
}

// Opt the transform kernels in to the largest dynamic shared memory the
// device allows next to their static shared memory (once per device).
template <typename K>
static cudaError_t allow_smem(K kernel, int optin) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}

cudaError_t configure_kernels() {
  static unsigned long long done = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 64 && (done >> dev & 1ull)) return cudaSuccess;
  int optin = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const cudaError_t r[18] = {allow_smem(k_xcond, optin), allow_smem(k_zinv<double>, optin), allow_smem(k_zinv<float>, optin),
                             allow_smem(k_zfwd<double>, optin), allow_smem(k_zfwd<float>, optin),
                             allow_smem(k_xprod<double>, optin), allow_smem(k_xprod<float>, optin), allow_smem(k_xprod2, optin),
                             allow_smem(k_xmask<double>, optin), allow_smem(k_xmask<float>, optin),
                             allow_smem(k_zinv_batch<double>, optin), allow_smem(k_zinv_batch<float>, optin),
                             allow_smem(k_zfwd_batch<double>, optin), allow_smem(k_zfwd_batch<float>, optin),
                             allow_smem(k_xprod_batch<double>, optin), allow_smem(k_xprod_batch<float>, optin),
                             allow_smem(k_xmask_batch<double>, optin), allow_smem(k_xmask_batch<float>, optin)};
  for (cudaError_t x : r)
    if (x != cudaSuccess) return x;
  if (dev < 64) done |= 1ull << dev;
  return cudaSuccess;
}

template void launch_zinv<double>(const ZJobs<double>&, const Dims&, const FftPlan&, int, cudaStream_t, int);
template void launch_zinv<float>(const ZJobs<float>&, const Dims&, const FftPlan&, int, cudaStream_t, int);
template void launch_zfwd<double>(const ZJobs<double>&, const Dims&, const FftPlan&, int, double, cudaStream_t, int);
template void launch_zfwd<float>(const ZJobs<float>&, const Dims&, const FftPlan&, int, double, cudaStream_t, int);
template void launch_xprod<double>(const ProdArgs<double>&, const Dims&, const FftPlan&, const FftPlan&, const double2*,
                                   cudaStream_t);
template void launch_xprod<float>(const ProdArgs<float>&, const Dims&, const FftPlan&, const FftPlan&, const double2*,
                                  cudaStream_t);
template void launch_xmask<double>(const MaskArgs<double>&, const Dims&, const FftPlan&, const double2*, cudaStream_t);
template void launch_xmask<float>(const MaskArgs<float>&, const Dims&, const FftPlan&, const double2*, cudaStream_t);
template void zpass_shape<double>(const ZJobs<double>&, const Dims&, int, dim3*, size_t*);
template void zpass_shape<float>(const ZJobs<float>&, const Dims&, int, dim3*, size_t*);
template void xprod_shape<double>(const ProdArgs<double>&, const Dims&, dim3*, size_t*);
template void xprod_shape<float>(const ProdArgs<float>&, const Dims&, dim3*, size_t*);
template void xmask_shape<double>(const MaskArgs<double>&, const Dims&, dim3*, size_t*);
template void xmask_shape<float>(const MaskArgs<float>&, const Dims&, dim3*, size_t*);
template void launch_zinv_batch<double>(const Batch<ZDesc<double>>&, size_t, cudaStream_t);
template void launch_zinv_batch<float>(const Batch<ZDesc<float>>&, size_t, cudaStream_t);
template void launch_zfwd_batch<double>(const Batch<ZDesc<double>>&, size_t, cudaStream_t);
template void launch_zfwd_batch<float>(const Batch<ZDesc<float>>&, size_t, cudaStream_t);
template void launch_xprod_batch<double>(const Batch<XDesc<double>>&, size_t, cudaStream_t);
template void launch_xprod_batch<float>(const Batch<XDesc<float>>&, size_t, cudaStream_t);
template void launch_xmask_batch<double>(const Batch<MDesc<double>>&, size_t, cudaStream_t);
template void launch_xmask_batch<float>(const Batch<MDesc<float>>&, size_t, cudaStream_t);

}  // namespace lh

