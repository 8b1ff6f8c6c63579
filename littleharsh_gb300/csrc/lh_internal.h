// lh_internal.h -- device state and kernel launchers shared by the C ABI
// (lh_capi.cu) and the kernels (lh_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "lh_fft.cuh"

struct lh_params;

namespace lh {

// Grid sizes.  Every level stores the wall bands' mode set (nkx x nz, the only
// one without variable-resolution bands).  With bands (Ngalx1 != Ngalx2,
// start.f90:95-118,1037-1145) the modes of the middle band's set are the long
// columns and span all levels; the others are short columns that live only in
// the wall bands (u levels 0..Nu1+1 and Nu2..nyu-1, v levels 0..Nv1+1 and
// Nv2..nyv-1, p levels 0..Nu1-1 and Nu2..nyp-1, end rows included) and are
// zero elsewhere.  A Dims passed to the plane kernels of the middle band has
// that band's nkx/nz/ngx/ngz/mp, and spitch/snz still describe the storage.
struct Dims {
  int nkx, nz, ngx, ngz;   // N1/2+1, N2, Ngal1, Ngal2 of the resolution the kernel works at
  int np;                  // stored spectral plane: spitch*snz complex
  int mp;                  // mixed plane (after the z transform): nkx*ngz complex
  int nyu, nyv, nyp;       // levels of the u, v and p grids
  int nn;                  // reference nn (= ny-2); u11 spans 0..nn+2
  int ju0;                 // global index of u level 0 (= jv0 = N(4,0)); p level 0 is ju0+1
  int spitch, snz;         // stored mode set: kx count (row pitch) and kz count
  int banded;              // 1: two resolutions (short and long columns)
  int nkx2, nz2;           // the middle band's mode set (long columns)
  int ngx2, ngz2;          // the middle band's physical points
  int Nu1, Nu2, Nv1, Nv2;  // level indices of N(4,1), N(4,2), N(3,1), N(3,2): the middle band's planes are
                           // u levels Nu1+1..Nu2 and v levels Nv1+1..Nv2
};

// Long column test for stored mode (i, kk) (columns_long_list, start.f90:1103-1117).
__host__ __device__ inline bool is_long(const Dims& d, int i, int kk) {
  if (!d.banded) return true;
  const int kz = kk < d.snz / 2 ? kk : kk - d.snz;
  return i < d.nkx2 && kz >= -(d.nz2 / 2) && kz < d.nz2 / 2;
}
// Where a column's y range (jlim, start.f90:1147-1175) puts level jj: 0 outside,
// 1 interior, 2 end row.
__host__ __device__ inline int lev_u(const Dims& d, bool lng, int jj) {
  if (lng) return (jj == 0 || jj == d.nyu - 1) ? 2 : 1;
  if (jj == 0 || jj == d.Nu1 + 1 || jj == d.Nu2 || jj == d.nyu - 1) return 2;
  return ((jj > 0 && jj <= d.Nu1) || (jj > d.Nu2 && jj < d.nyu - 1)) ? 1 : 0;
}
__host__ __device__ inline int lev_v(const Dims& d, bool lng, int jj) {
  if (lng) return (jj == 0 || jj == d.nyv - 1) ? 2 : 1;
  if (jj == 0 || jj == d.Nv1 + 1 || jj == d.Nv2 || jj == d.nyv - 1) return 2;
  return ((jj > 0 && jj <= d.Nv1) || (jj > d.Nv2 && jj < d.nyv - 1)) ? 1 : 0;
}
// p level jp (global j = ju0 + 1 + jp) inside the column
__host__ __device__ inline bool lev_p(const Dims& d, bool lng, int jp) {
  return lng || jp < d.Nu1 || jp >= d.Nu2;
}
// the middle band's planes
__host__ __device__ inline bool coarse_u(const Dims& d, int jj) { return d.banded && jj > d.Nu1 && jj <= d.Nu2; }
__host__ __device__ inline bool coarse_v(const Dims& d, int jj) { return d.banded && jj > d.Nv1 && jj <= d.Nv2; }

// Read-only per-run tables in device memory.
struct Tables {
  const double* kx;    // [nkx] alp*i
  const double* kz;    // [nz]  signed bet*kz
  const double* k2x;   // [nkx] -(alp i)^2
  const double* k2z;   // [nz]
  const double* d2u;   // [nyu][3] dyu2i
  const double* d2v;   // [nyv][3] dyv2i
  const double* cu;    // [nyu] ddthetavi*dthdyu
  const double* cv;    // [nyv] ddthetavi*dthdyv
  const double* wc;    // [nyu] weight of face j in the centre-j interpolation of v
  const double* wf;    // [nyv] weight of centre j+1 in the face-j interpolation of u, w
  const double* dyc;   // [nyu] 1/(yv(j)-yv(j-1)) at centres, for the CFL number
  const double* dyvw;  // [nn+2] yv(j)-yv(j-1), j = 1..nn+1 at index j (flow rate)
  const double* lu_u;  // [3 kRK][3][nyu] Helmholtz LU (a1, 1/diag, scaled a3), u grid, long columns
  const double* lu_v;  // [3 kRK][3][nyv] same, v grid
  const double* lu_u1; // [3 kRK][3][nyu] short columns' bottom band (levels 0..Nu1+1; with bands only)
  const double* lu_u3; // [3 kRK][3][nyu] short columns' top band (levels Nu2..nyu-1)
  const double* lu_v1; // [3 kRK][3][nyv] (levels 0..Nv1+1)
  const double* lu_v3; // [3 kRK][3][nyv] (levels Nv2..nyv-1)
  const double* u11;   // [3 kRK][nn+3] unit-gradient response of mode (0,0)
  const double* iaxz;  // [3 kRK][np] 1/axz = 1/(1 - beta_k (k2x + k2z)) per column
  const double* dg1;   // [nyp] pressure LU lower diagonal (column independent)
  const double* dg2;   // [nyp][np] pressure LU 1/diag per column
  const double* dg3;   // [nyp][np] pressure LU scaled upper diagonal per column
  // kx, kz, cu, cv rounded to FP32 once (the mixed form's nonlinear term combines its FP32 spectra with them;
  // on this part a conversion costs about as much as an FP64 instruction)
  const float* kxf;
  const float* kzf;
  const float* cuf;
  const float* cvf;
};

// Canopy forcing: processed planes of one field.
struct IbSet {
  int nplanes;            // planes of the u grid (u1, u3) or v grid (u2)
  const int* levels;      // [nplanes] level index on the field's own grid
  const uint8_t* mask;    // [nplanes][ngz][ngx] 1 = solid
  const int* tipslot;     // [nplanes] -1, or index of the plane's y-Laplacian in the tip buffer
};

// Scalars kept on the device so a whole step can run as one CUDA graph.
struct DevScalars {
  double mpgx;   // mean pressure gradient
  double QxT;    // target flow rate
  double Qx;     // last flow rate seen by the correction
  unsigned long long cflbits;  // max CFL number (bit pattern of a non-negative double)
  int err;       // sticky error bits (kErr*), cleared when fields are uploaded
};
constexpr int kErrNonFinite = 1;  // the pressure solve produced a NaN or an infinity

// Transform job for the z passes: nlev planes; plane y of the job reads
// level (levels ? levels[y] : lev0 + y) of `spec` and uses mix plane y.
template <typename R>
struct ZJob {
  const double2* spec_in;   // z-inverse: spectral source
  double2* spec_out;        // z-forward: spectral destination
  cpx_t<R>* mix;            // mixed planes, contiguous per job
  const int* levels;
  int lev0, nlev;
  int out32;                // z-forward: write FP32 spectra (cpx_t<R>) to spec_out instead of FP64
  int nomean;               // z-inverse: leave the (0,0) mode out (the mixed form carries the mean profile apart)
};

constexpr int kMaxJobs = 12;
template <typename R>
struct ZJobs {
  ZJob<R> j[kMaxJobs];
  int njobs, maxlev;
};

// Launchers (lh_kernels.cu).  All are asynchronous on `st`.
template <typename R>
void launch_zinv(const ZJobs<R>& jobs, const Dims& d, const FftPlan& pz, int tx, cudaStream_t st, int threads = 256);
template <typename R>
void launch_zfwd(const ZJobs<R>& jobs, const Dims& d, const FftPlan& pz, int tx, double scale, cudaStream_t st,
                 int threads = 256);

template <typename R>
struct ProdArgs {
  const cpx_t<R>* mu;   // [nyu] mixed planes of u (levels 1..nyu-2 used)
  const cpx_t<R>* mw;   // [nyu] w
  const cpx_t<R>* mv;   // [nyv] v (levels 1..nyv-2 used)
  cpx_t<R>* out[6];     // uu, uw, ww, vv on [nyu]; uv, vw on [nyv]
  const double* wc;
  const double* wf;
  const double* dyc;
  double dxi, dzi;
  DevScalars* sc;       // CFL maximum accumulated here when want_cfl
  int want_cfl;
  int chunk;
  int split;            // 1: the face pair is transformed after the centre pairs, through two buffer vectors
  int threads;          // threads per CTA of the stand-alone launch (128 or 256; the batched launch uses 256)
  int rows;             // z rows per CTA of the stand-alone launch: 2 runs two rows' transforms in lockstep
                        // (FP32, unsplit, ngz even; the same arithmetic per row); otherwise 1
  // levels this launch forms products on (a band's planes): centres c_lo..c_hi, faces f_lo..f_hi
  int c_lo, c_hi, f_lo, f_hi;
  // mixed form: mu, mw hold the fluctuations u' = u - U(y), w' = w - W(y) (the z-inverse left the (0,0) modes
  // out) and the products are formed as u'(2U + u'), u'(W + w') + U w', w'(2W + w'), (U_f + u'_f) v,
  // (W_f + w'_f) v with the level means U, W read from the (0,0) modes of us, ws (nps apart): the FP32 values
  // never hold U^2 beside products ten to a hundred times smaller.  The left-out U^2, UW reach only the (0,0)
  // modes of uu, uw, ww, of which the nonlinear term takes no derivative.
  int mean_split;
  const double2 *us, *ws;
  int nps;
};
template <typename R>
void launch_xprod(const ProdArgs<R>& a, const Dims& d, const FftPlan& ph, const FftPlan& pf, const double2* rtw,
                  cudaStream_t st);

template <typename R>
struct MaskArgs {
  cpx_t<R>* mix;          // all processed planes, contiguous: [nplanes_total][ngz][nkx]
  const cpx_t<R>* lymix;  // tip planes' y-Laplacian
  const uint8_t* mask[3];
  const int* tipslot[3];
  int nplanes[3];
  double beta;
};
template <typename R>
void launch_xmask(const MaskArgs<R>& a, const Dims& d, const FftPlan& ph, const double2* rtw, cudaStream_t st);

struct AsmArgs {
  const double2 *u1, *u2, *u3, *p;
  double2 *n1, *n2, *n3;     // in: Nu of the previous substage, out: Nu of this one
  double2 *r1, *r2, *r3;     // out: right-hand sides divided by axz
  // product spectra uu, uw, ww, vv (centres), uv, vw (faces): FP64, or FP32 in the mixed form (p32 set)
  const double2* p64[6];
  const float2* p32[6];
  double2* lytip;            // y-Laplacian of the tip planes [6][np]
  int tipu[2], tipv[2];      // level indices of the tip planes (u grid, v grid) or -1
  const DevScalars* sc;
  double C1, C2, d, g, dt, beta;
  int k;                     // substage index 0..2 (selects 1/axz)
};
void launch_assemble(const AsmArgs& a, const Dims& d, const Tables& t, cudaStream_t st);

void launch_vsolve(double2* r1, double2* r2, double2* r3, double2* u1, double2* u2, double2* u3,
                   const Dims& d, const Tables& t, int k, cudaStream_t st);
void launch_flowrate(double2* u1, DevScalars* sc, const Dims& d, const Tables& t, int k, double Qx1, cudaStream_t st);
void launch_build_dg(double* dg2, double* dg3, const double* rows, const Dims& d, const Tables& t, double pin,
                     cudaStream_t st);
// sc may be NULL; otherwise kErrNonFinite is or-ed into sc->err when a corrected value is not finite
void launch_psolve(double2* u1, double2* u2, double2* u3, double2* p, double2* psi, const Dims& d,
                   const Tables& t, double dtirk, double dtrk, double gwb, double gwt, DevScalars* sc,
                   cudaStream_t st);
void launch_divergence(const double2* u1, const double2* u2, const double2* u3, double2* div, const Dims& d,
                       const Tables& t, cudaStream_t st);
void launch_absmax(const double2* x, size_t n, DevScalars* sc, cudaStream_t st);
void launch_transpose(const double2* src, double2* dst, int rows, int cols, cudaStream_t st);
// dst[j] = src[j * stride], j < n (one strided column gathered into contiguous scratch)
void launch_gather_col(const double2* src, size_t stride, int n, double2* dst, cudaStream_t st);
void launch_spectra(const double2* u1, const double2* u2, const double2* u3, const double2* p, double* sp,
                    const Dims& d, const Tables& t, cudaStream_t st);
// vc, wf: nyu and nyv staging planes; om: nyv staging planes (omega_x)
void launch_stats(const double2* u1, const double2* u2, const double2* u3, const double2* p, double2* vc,
                  double2* wf, double2* om, double* acc, const Dims& d, const Tables& t, cudaStream_t st);
// Conditional statistics pass over one chunk of wall-band planes (grids g: 0 u, 1 v, 2 p).
struct CondArgs {
  const double2* mix[3][3];  // mixed planes per grid and field (u: u, w, v at centres; v: v, w, omega_x at faces;
                             // p: p)
  double* out[3];            // accumulators per grid: [quantity][j1][kin][i]
  double* outw;              // the v grid's omega_x accumulators: [2][j1][kin][i]
  int nj[3];                 // planes of this chunk per grid
  int njtot[3];              // planes per grid in total
  int j0;                    // first j1 of the chunk
  int dnx, dnz, ntx, ntz;
};
// v at every centre and w at every face (zero on ghost centres and wall faces); om (may be NULL): omega_x at
// every face
void launch_stage_itp(const double2* u2, const double2* u3, double2* vc, double2* wf, double2* om, const Dims& d,
                      const Tables& t, cudaStream_t st);
void launch_xcond(const CondArgs& a, const Dims& d, const FftPlan& ph, const double2* rtw, cudaStream_t st);
// ---------------------------------------------------------------------------
// Batched launches: one launch of a kernel kind covers the work of several
// independent solvers (an ensemble).  The members' arguments travel as one
// kernel parameter (Batch<D>, under the 32 KB parameter limit), read from the
// constant bank like a single launch's; member m owns the blocks start[m] ..
// start[m+1]-1 of the launch's one-dimensional grid, laid out as its own
// gx x gy x gz grid would be.  The arithmetic of a block is that of the
// single-solver launch, so the results are bit for bit the same.
// ---------------------------------------------------------------------------
constexpr int kMaxBatch = 32;   // members per batched launch (larger ensembles take several)
template <typename R>
struct ZDesc {                  // z-inverse or z-forward
  ZJobs<R> jobs;
  Dims d;
  FftPlan p;
  double scale;
  int tx, gx, gy, gz;
};
template <typename R>
struct XDesc {                  // x pass with the products
  ProdArgs<R> a;
  Dims d;
  FftPlan ph, pf;
  const double2* rtw;
  int gx, gy;
};
template <typename R>
struct MDesc {                  // canopy forcing x pass
  MaskArgs<R> a;
  Dims d;
  FftPlan ph;
  const double2* rtw;
  int gx, gy;
};
struct ADesc {                  // right-hand-side assembly
  AsmArgs a;
  Dims d;
  Tables t;
  int gx, gy;
};
struct VDesc {                  // velocity Thomas sweeps
  double2 *r1, *r2, *r3, *u1, *u2, *u3;
  Dims d;
  Tables t;
  int k, gx, gy;
};
struct FDesc {                  // flow-rate correction (one block)
  double2* u1;
  DevScalars* sc;
  Dims d;
  Tables t;
  int k;
  double Qx1;
};
struct PDesc {                  // pressure solve and correction
  double2 *u1, *u2, *u3, *p, *psi;
  Dims d;
  Tables t;
  double dtirk, dtrk, gwb, gwt;
  DevScalars* sc;
  int gx;
};
template <typename D>
struct Batch {
  int n;                      // members in this launch
  int start[kMaxBatch + 1];   // first block of each member, start[n] = total blocks
  D desc[kMaxBatch];
};
static_assert(sizeof(Batch<ZDesc<double>>) < 32700 && sizeof(Batch<XDesc<double>>) < 32700 &&
                  sizeof(Batch<ADesc>) < 32700 && sizeof(Batch<MDesc<double>>) < 32700,
              "a batch must fit the kernel parameter limit");
// Launchers of the batched kernels (start[] filled from the members' gx*gy*gz; smem: the largest dynamic shared
// memory any member needs).
template <typename R>
void launch_zinv_batch(const Batch<ZDesc<R>>& b, size_t smem, cudaStream_t st);
template <typename R>
void launch_zfwd_batch(const Batch<ZDesc<R>>& b, size_t smem, cudaStream_t st);
template <typename R>
void launch_xprod_batch(const Batch<XDesc<R>>& b, size_t smem, cudaStream_t st);
template <typename R>
void launch_xmask_batch(const Batch<MDesc<R>>& b, size_t smem, cudaStream_t st);
void launch_assemble_batch(const Batch<ADesc>& b, bool fp32_products, cudaStream_t st);
void launch_vsolve_batch(const Batch<VDesc>& b, cudaStream_t st);
void launch_flowrate_batch(const Batch<FDesc>& b, cudaStream_t st);
void launch_psolve_batch(const Batch<PDesc>& b, cudaStream_t st);
// Grid and dynamic shared memory of the single launches (what the batched ones reproduce per member; a zero
// grid means no launch).
template <typename R>
void zpass_shape(const ZJobs<R>& jobs, const Dims& d, int tx, dim3* grid, size_t* smem);
template <typename R>
void xprod_shape(const ProdArgs<R>& a, const Dims& d, dim3* grid, size_t* smem);
template <typename R>
void xmask_shape(const MaskArgs<R>& a, const Dims& d, dim3* grid, size_t* smem);

cudaError_t configure_kernels();
// Measured FP64 FMA throughput of the current device in TFLOP/s (FMA = 2 flops), best of three timed
// launches of a probe kernel; -1 on a CUDA error.  nsm_out (may be NULL) receives the SM count.
double fp64_probe_tflops(int* nsm_out);

// Grid sizes of a parameter block, with the checks lh_init makes (lh_capi.cu): LH_OK, or an LH_E* code and
// the reason in *why.
int make_dims(const ::lh_params* prm, Dims* out, std::string* why);

// Message returned by lh_last_error(NULL) on this thread (lh_capi.cu).
void set_init_error(const char* msg);

}  // namespace lh
