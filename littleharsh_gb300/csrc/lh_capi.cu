// lh_capi.cu -- the C ABI of include/littleharsh.h.
//
// One handle owns one solver on one device: the read-only tables, the
// device-resident fields and the scratch the substage pipeline needs.  A full
// RK3 step (three substages, littleharsh.f90:164-190) is enqueued on the
// handle's stream, captured once into a CUDA graph and replayed; nothing in the
// step synchronises with the host.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/littleharsh.h"
#include "lh_internal.h"

using namespace lh;

namespace {

constexpr long double kPi = 3.141592653589793238462643383279502884L;
thread_local std::string g_init_error;

struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
};

// One transform length with its device tables.
struct PlanStore {
  FftPlan plan{};
  DevBuf perm, tw64, tw32;
};

}  // namespace

struct lh_handle {
  int device = 0;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  int precision = LH_PREC_FP64;
  Dims d{};
  Tables t{};
  lh_params prm{};
  // host copies
  std::vector<double> yu, yv, dthdyu, dthdyv, dyu2i, dyv2i;
  std::vector<double> kx, kz, k2x, k2z;
  double gw[3][2]{};
  double Re = 0, alp = 0, bet = 0, Lx = 0, Lz = 0, dtv = 0;
  double aRK[3]{}, bRK[3]{}, gRK[3]{}, cRK[3]{}, dRK[3]{};
  double Qx1[3]{};
  int nibu = 0, nibv = 0;
  int tipu[2]{-1, -1}, tipv[2]{-1, -1};
  // device memory
  std::vector<void*> allocs;
  double2 *u1 = nullptr, *u2 = nullptr, *u3 = nullptr, *p = nullptr;
  double2 *n1 = nullptr, *n2 = nullptr, *n3 = nullptr;
  double2 *r1 = nullptr, *r2 = nullptr, *r3 = nullptr;
  double2 *puu = nullptr, *puw = nullptr, *pww = nullptr, *pvv = nullptr, *puv = nullptr, *pvw = nullptr;
  double2 *psi = nullptr, *lytip = nullptr, *stage = nullptr;
  void *mixu = nullptr, *mixw = nullptr, *mixv = nullptr, *mixp[6] = {}, *mixib = nullptr, *mixly = nullptr;
  int *ibu_lev = nullptr, *ibv_lev = nullptr, *ibu_tip = nullptr, *ibv_tip = nullptr, *ibw_tip = nullptr;
  uint8_t *ibu_mask = nullptr, *ibv_mask = nullptr;
  double* spec = nullptr;  // spectra accumulators
  int nspec = 0;
  double* stat = nullptr;  // plane statistics accumulators, 13 rows of max(nyu, nyv)
  int nstat = 0;
  // conditional statistics: planes per grid, tile size, accumulators, level lists (both walls interleaved)
  int nju = 0, njv = 0, njp = 0, dnx = 0, dnz = 0, ncond = 0;
  double* cond = nullptr;
  int *cond_ul = nullptr, *cond_vl = nullptr, *cond_pl = nullptr;
  double* tabs = nullptr;  // lu_u, lu_v, u11 (rewritten when dt changes)
  DevScalars* sc = nullptr;
  PlanStore pz, ph, pf;  // z (Ngalz), x half length (Ngalx/2), x full length (Ngalx)
  double2* rtw = nullptr;
  PlanStore pz2, ph2, pf2;  // the same for the middle band (bands only)
  double2* rtw2 = nullptr;
  Dims dmid{};              // the middle band's plane geometry (bands only)
  int tx = 8, chunk = 16;
  int xsplit = 0;  // x-pass: face pair transformed on its own (smaller shared-memory footprint)
  int xthreads = 256;  // x-pass: threads per CTA (128 or 256)
  int zthreads = 256;  // z passes of the nonlinear term and the canopy forcing: threads per CTA (128 or 256)
  int xrows = 1;       // x-pass: z rows per CTA (2: the mixed form's two-row lockstep kernel)
  // state
  double t_now = 0, dt = 0;
  bool have_fields = false, have_dt = false;
  long long iter = 0;
  cudaGraphExec_t graph = nullptr;
  unsigned long long graph_gen = 0;  // bumped whenever captured launch arguments (dt) change
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0;
  // step monitor (lh_set_monitor): max |div| checked against maxerr every mon_every steps (0 = off)
  double mon_maxerr = 0;
  int mon_every = 0;
  double last_divmax = -1;
  int launches_per_step = 0;
  // per-launch timing (lh_profile_step): kind of each launch and the event recorded after it
  bool profiling = false;
  std::vector<int> prof_kind;
  std::vector<cudaEvent_t> prof_ev;
  std::string err;
};

namespace {

int fail(lh_handle* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  else g_init_error = buf;
  return code;
}

#define CU(h, call)                                                                        \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return fail((h), LH_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// Kinds of launches reported by lh_profile_step.
enum { K_ZINV, K_XPROD, K_ZFWD, K_ASSEMBLE, K_IB_ZINV, K_IB_XMASK, K_IB_ZFWD, K_VSOLVE, K_FLOWRATE, K_PSOLVE, K_NKINDS };

void mark(lh_handle* h, int kind) {
  if (!h->profiling) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, h->st);
  h->prof_kind.push_back(kind);
  h->prof_ev.push_back(e);
}

template <typename T>
int dalloc(lh_handle* h, T** out, size_t count) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T) + 16);
  if (e != cudaSuccess) return fail(h, LH_ENOMEM, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
  h->allocs.push_back(p);
  cudaMemsetAsync(p, 0, count * sizeof(T) + 16, h->st);
  *out = static_cast<T*>(p);
  return LH_OK;
}

template <typename T>
int upload(lh_handle* h, T** out, const std::vector<T>& v) {
  int rc = dalloc(h, out, v.size());
  if (rc) return rc;
  CU(h, cudaMemcpyAsync(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, h->st));
  return LH_OK;
}

// Stages of a DIT sequence for length n: radix 4 first (stage 0 has no
// twiddles, which saves the most on radix 4), then 2, radix 3 last (so that
// the last stage splits the output in thirds, which the z-forward can prune).
int build_plan(lh_handle* h, PlanStore& ps, int n, int keep_half) {
  FftPlan& P = ps.plan;
  std::memset(&P, 0, sizeof P);
  P.n = n;
  int m = n, n4 = 0, n2 = 0, n3 = 0;
  while (m % 4 == 0) { m /= 4; ++n4; }
  while (m % 2 == 0) { m /= 2; ++n2; }
  while (m % 3 == 0) { m /= 3; ++n3; }
  if (m != 1) return fail(h, LH_EFFT, "transform length %d does not factor into 2, 3 and 4", n);
  int s = 0;
  for (int i = 0; i < n4; ++i) P.rad[s++] = 4;
  for (int i = 0; i < n2; ++i) P.rad[s++] = 2;
  for (int i = 0; i < n3; ++i) P.rad[s++] = 3;
  if (s > kMaxStages) return fail(h, LH_EFFT, "transform length %d needs too many stages", n);
  P.ns = s;
  int L = 1;
  for (int i = 0; i < s; ++i) {
    L *= P.rad[i];
    P.len[i] = L;
    P.mdiv[i] = fdiv_mult((unsigned)(L / P.rad[i]));
    P.qdiv[i] = fdiv_mult((unsigned)(n / P.rad[i]));
  }
  // the output slots a truncation keeps are [0, keep_half) and [n - keep_half, n)
  P.prune_mid = (s > 0 && P.rad[s - 1] == 3 && keep_half > 0 && keep_half * 3 == n) ? 1 : 0;
  std::vector<int> perm(n);
  for (int f = 0; f < n; ++f) {
    int pos = 0, x = f, len = n;
    for (int i = s - 1; i >= 0; --i) {
      const int r = P.rad[i], sub = len / r;
      pos += (x % r) * sub;
      x /= r;
      len = sub;
    }
    perm[f] = pos;
  }
  std::vector<double2> t64(n);
  std::vector<float2> t32(n);
  for (int k = 0; k < n; ++k) {
    const long double a = 2.0L * kPi * (long double)k / (long double)n;
    t64[k] = double2{(double)cosl(a), -(double)sinl(a)};
    t32[k] = float2{(float)t64[k].x, (float)t64[k].y};
  }
  int* dperm;
  double2* d64;
  float2* d32;
  int rc;
  if ((rc = upload(h, &dperm, perm)) || (rc = upload(h, &d64, t64)) || (rc = upload(h, &d32, t32))) return rc;
  P.perm = dperm;
  P.tw64 = d64;
  P.tw32 = d32;
  return LH_OK;
}

size_t field_elems(const lh_handle* h, char grid) {
  const int ny = grid == 'u' ? h->d.nyu : (grid == 'v' ? h->d.nyv : h->d.nyp);
  return (size_t)ny * h->d.np;
}

// LU_build + LU_dec (tridLU_3D_IB.f90:427-493,601-640) over levels lo..hi of
// one grid (coefficients c = dyu2i or dyv2i per level), boundary rows
// [1, gwl] and [gwh, 1] (u) or identity rows (v: gwl = gwh = 0).
void helm_lu_host(double* a1, double* a2, double* a3, const std::vector<double>& c, int lo, int hi, double beta,
                  double gwl, double gwh) {
  a1[lo] = 0.0; a2[lo] = 1.0; a3[lo] = gwl;
  for (int j = lo + 1; j < hi; ++j) {
    a1[j] = -beta * c[3 * j];
    a2[j] = 1.0 - beta * (c[3 * j + 1]);
    a3[j] = -beta * c[3 * j + 2];
  }
  a1[hi] = gwh; a2[hi] = 1.0; a3[hi] = 0.0;
  a2[lo] = 1.0 / a2[lo];
  for (int j = lo + 1; j <= hi; ++j) {
    a3[j - 1] = a3[j - 1] * a2[j - 1];
    a2[j] = 1.0 / (a2[j] - a1[j] * a3[j - 1]);
  }
}

// Helmholtz LU for the three substages (long columns over the whole channel
// with band 2's gridweighting; with bands also the short columns' bottom and
// top bands with bands 1 and 3's) and the unit-gradient response of mode
// (0,0) (LUsol0, :398-424) for the current dt.
int build_dt_tables(lh_handle* h) {
  const Dims& d = h->d;
  const int nyu = d.nyu, nyv = d.nyv, n0 = d.nn + 3;
  const size_t np = d.np;
  const int nb = d.banded ? 3 : 1;  // LU sets per grid: long (, bottom, top)
  std::vector<double> all(nb * 9 * (size_t)nyu + nb * 9 * (size_t)nyv + 3 * n0 + 3 * np);
  double* luu = all.data();
  double* luv = luu + 9 * nyu;
  double* luu1 = luv + 9 * nyv;       // used with bands only
  double* luu3 = luu1 + 9 * nyu;
  double* luv1 = luu3 + 9 * nyu;
  double* luv3 = luv1 + 9 * nyv;
  double* u11 = all.data() + nb * 9 * (size_t)nyu + nb * 9 * (size_t)nyv;
  double* iaxz = u11 + 3 * n0;
  for (int k = 0; k < 3; ++k) {
    const double beta = h->bRK[k] * h->dt / h->Re;
    for (int grid = 0; grid < 2; ++grid) {
      const int ny = grid == 0 ? nyu : nyv;
      const std::vector<double>& c = grid == 0 ? h->dyu2i : h->dyv2i;
      double* a1 = (grid == 0 ? luu : luv) + (size_t)k * 3 * ny;
      helm_lu_host(a1, a1 + ny, a1 + 2 * ny, c, 0, ny - 1, beta, grid == 0 ? h->gw[1][0] : 0.0,
                   grid == 0 ? h->gw[1][1] : 0.0);
      if (d.banded) {
        const int e1 = grid == 0 ? d.Nu1 + 1 : d.Nv1 + 1, s3 = grid == 0 ? d.Nu2 : d.Nv2;
        double* b1 = (grid == 0 ? luu1 : luv1) + (size_t)k * 3 * ny;
        double* b3 = (grid == 0 ? luu3 : luv3) + (size_t)k * 3 * ny;
        helm_lu_host(b1, b1 + ny, b1 + 2 * ny, c, 0, e1, beta, grid == 0 ? h->gw[0][0] : 0.0,
                     grid == 0 ? h->gw[0][1] : 0.0);
        helm_lu_host(b3, b3 + ny, b3 + 2 * ny, c, s3, ny - 1, beta, grid == 0 ? h->gw[2][0] : 0.0,
                     grid == 0 ? h->gw[2][1] : 0.0);
      }
    }
    // LU_build0 on global indices 0..nn+2
    const int nn = d.nn, ju0 = d.ju0;
    std::vector<double> b1(n0), b2(n0), b3(n0);
    b1[0] = 0.0; b2[0] = 1.0; b3[0] = h->gw[1][0];
    for (int j = 1; j <= nn + 1; ++j) {
      const double* c = &h->dyu2i[3 * (j - ju0)];
      b1[j] = -beta * c[0];
      b2[j] = 1.0 - beta * c[1];
      b3[j] = -beta * c[2];
    }
    b1[nn + 2] = h->gw[1][1]; b2[nn + 2] = 1.0; b3[nn + 2] = 0.0;
    b2[0] = 1.0 / b2[0];
    for (int j = 1; j < n0; ++j) {
      b3[j - 1] = b3[j - 1] * b2[j - 1];
      b2[j] = 1.0 / (b2[j] - b1[j] * b3[j - 1]);
    }
    double* x = u11 + (size_t)k * n0;
    const double bdt = -h->dRK[k] * h->dt;
    x[0] = 0.0;
    for (int j = 1; j <= nn + 1; ++j) x[j] = bdt;
    x[nn + 2] = 0.0;
    x[0] = x[0] * b2[0];
    for (int j = 1; j < n0; ++j) x[j] = (x[j] - b1[j] * x[j - 1]) * b2[j];
    for (int j = n0 - 2; j >= 0; --j) x[j] = x[j] - b3[j] * x[j + 1];
    // flowrateRe sees u11(0:) as u(1:) (sequence association at littleharsh.f90:474)
    double Q = 0.0;
    for (int j = 1; j <= nn + 1; ++j) Q = Q + (h->yv[j - ju0] - h->yv[j - 1 - ju0]) * x[j - 1];
    h->Qx1[k] = Q;
    // 1/axz per column (LU_build, tridLU_3D_IB.f90:484-491)
    for (size_t col = 0; col < np; ++col) {
      const int i = (int)(col % d.nkx), kk = (int)(col / d.nkx);
      iaxz[(size_t)k * np + col] = 1.0 / (1.0 - beta * (h->k2x[i] + h->k2z[kk]));
    }
  }
  if (!h->tabs) {
    int rc = dalloc(h, &h->tabs, all.size());
    if (rc) return rc;
  }
  CU(h, cudaMemcpyAsync(h->tabs, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice, h->st));
  h->t.lu_u = h->tabs;
  h->t.lu_v = h->tabs + 9 * nyu;
  h->t.lu_u1 = d.banded ? h->tabs + 9 * nyu + 9 * nyv : h->t.lu_u;
  h->t.lu_u3 = d.banded ? h->t.lu_u1 + 9 * nyu : h->t.lu_u;
  h->t.lu_v1 = d.banded ? h->t.lu_u3 + 9 * nyu : h->t.lu_v;
  h->t.lu_v3 = d.banded ? h->t.lu_v1 + 9 * nyv : h->t.lu_v;
  h->t.u11 = h->tabs + nb * 9 * (size_t)nyu + nb * 9 * (size_t)nyv;
  h->t.iaxz = h->t.u11 + 3 * n0;
  CU(h, cudaStreamSynchronize(h->st));
  return LH_OK;
}

// The plane work of the nonlinear term per band: which geometry and transforms
// a band's planes use, and the centre and face levels it forms products on
// (planelim, start.f90:1336-1383).
struct BandLaunch {
  const Dims* d;
  const FftPlan *pz, *ph, *pf;
  const double2* rtw;
  int c_lo, c_hi, f_lo, f_hi;
};
int band_launches(const lh_handle* h, BandLaunch* out) {
  const Dims& d = h->d;
  const BandLaunch fine{&d, &h->pz.plan, &h->ph.plan, &h->pf.plan, h->rtw, 0, 0, 0, 0};
  if (!d.banded) {
    out[0] = fine;
    out[0].c_lo = 1; out[0].c_hi = d.nyu - 2; out[0].f_lo = 1; out[0].f_hi = d.nyv - 2;
    return 1;
  }
  out[0] = fine;
  out[0].c_lo = 1; out[0].c_hi = d.Nu1; out[0].f_lo = 1; out[0].f_hi = d.Nv1;
  out[1] = BandLaunch{&h->dmid, &h->pz2.plan, &h->ph2.plan, &h->pf2.plan, h->rtw2, d.Nu1 + 1, d.Nu2, d.Nv1 + 1, d.Nv2};
  out[2] = fine;
  out[2].c_lo = d.Nu2 + 1; out[2].c_hi = d.nyu - 2; out[2].f_lo = d.Nv2 + 1; out[2].f_hi = d.nyv - 2;
  return 3;
}

// The nonlinear term's plane work for one band: z-inverse of the levels the band's products need, products,
// z-forward of the band's product planes, with the geometry and transforms of the band's planes.
template <typename R>
struct NlBand {
  const Dims* d;
  const FftPlan *pz, *ph, *pf;
  const double2* rtw;
  ZJobs<R> zi, zf;
  ProdArgs<R> xp;
};

template <typename R>
int nl_bands(const lh_handle* h, NlBand<R>* out) {
  using T2 = cpx_t<R>;
  const Dims& d = h->d;
  BandLaunch bl[3];
  const int nbl = band_launches(h, bl);
  for (int b = 0; b < nbl; ++b) {
    const BandLaunch& B = bl[b];
    const Dims& db = *B.d;
    NlBand<R>& o = out[b];
    o.d = B.d; o.pz = B.pz; o.ph = B.ph; o.pf = B.pf; o.rtw = B.rtw;
    const int L0 = std::min(B.c_lo, B.f_lo + 1), L1 = std::max(B.c_hi, B.f_hi + 1);
    {
      const int ul = std::max(1, L0 - 1), uh = std::min(d.nyu - 2, L1);
      const int vl = std::max(1, L0 - 1), vh = std::min(d.nyv - 2, L1);
      ZJobs<R> J{};
      J.j[0] = ZJob<R>{h->u1, nullptr, (T2*)h->mixu + (size_t)ul * db.mp, nullptr, ul, uh - ul + 1};
      J.j[1] = ZJob<R>{h->u3, nullptr, (T2*)h->mixw + (size_t)ul * db.mp, nullptr, ul, uh - ul + 1};
      J.j[2] = ZJob<R>{h->u2, nullptr, (T2*)h->mixv + (size_t)vl * db.mp, nullptr, vl, std::max(0, vh - vl + 1)};
      // the mixed form transforms the fluctuations of u and w; the product pass adds the level means back
      // outside the FP32 transforms (ProdArgs::mean_split)
      J.j[0].nomean = J.j[1].nomean = sizeof(R) == 4;
      J.njobs = 3;
      J.maxlev = uh - ul + 1;
      o.zi = J;
    }
    {
      ProdArgs<R> a{};
      a.mu = (const T2*)h->mixu;
      a.mw = (const T2*)h->mixw;
      a.mv = (const T2*)h->mixv;
      for (int i = 0; i < 6; ++i) a.out[i] = (T2*)h->mixp[i];
      a.wc = h->t.wc; a.wf = h->t.wf; a.dyc = h->t.dyc;
      a.dxi = db.ngx / h->Lx; a.dzi = db.ngz / h->Lz;
      a.sc = h->sc; a.want_cfl = 0; a.chunk = h->chunk; a.split = h->xsplit; a.threads = h->xthreads;
      a.rows = (sizeof(R) == 4 && h->xrows == 2 && !h->xsplit && db.ngz % 2 == 0) ? 2 : 1;
      a.c_lo = B.c_lo; a.c_hi = B.c_hi; a.f_lo = B.f_lo; a.f_hi = B.f_hi;
      a.mean_split = sizeof(R) == 4;
      a.us = h->u1; a.ws = h->u3; a.nps = d.np;
      o.xp = a;
    }
    {
      ZJobs<R> J{};
      double2* outs[6] = {h->puu, h->puw, h->pww, h->pvv, h->puv, h->pvw};
      for (int i = 0; i < 6; ++i) {
        const int lo = i < 4 ? B.c_lo : B.f_lo, hi = i < 4 ? B.c_hi : B.f_hi;
        J.j[i] = ZJob<R>{nullptr, outs[i], (T2*)h->mixp[i] + (size_t)lo * db.mp, nullptr, lo, std::max(0, hi - lo + 1)};
        J.j[i].out32 = sizeof(R) == 4;  // the mixed form keeps its product spectra in FP32
      }
      J.njobs = 6;
      J.maxlev = std::max(B.c_hi - B.c_lo + 1, B.f_hi - B.f_lo + 1);
      o.zf = J;
    }
  }
  return nbl;
}

// The nonlinear term's plane work, one band at a time (one band without
// variable resolution).  The flags select parts (the autotuner times them
// separately); a substage runs all three.
template <typename R>
void enqueue_nonlinear(lh_handle* h, cudaStream_t st, bool zinv, bool xprod, bool zfwd) {
  NlBand<R> bl[3];
  const int nbl = nl_bands<R>(h, bl);
  for (int b = 0; b < nbl; ++b) {
    const NlBand<R>& B = bl[b];
    if (zinv) {
      launch_zinv<R>(B.zi, *B.d, *B.pz, h->tx, st, h->zthreads);
      mark(h, K_ZINV);
    }
    if (xprod) {
      launch_xprod<R>(B.xp, *B.d, *B.ph, *B.pf, B.rtw, st);
      mark(h, K_XPROD);
    }
    if (zfwd) {
      launch_zfwd<R>(B.zf, *B.d, *B.pz, h->tx, 1.0 / B.d->ngz, st, h->zthreads);
      mark(h, K_ZFWD);
    }
  }
}

// One timed pass of the autotuner: the z passes and/or the product pass of the
// nonlinear term, best of two, in milliseconds (negative on a CUDA error).
template <typename R>
float time_parts(lh_handle* h, bool z, bool x, cudaEvent_t e0, cudaEvent_t e1) {
  float best = 1e30f;
  for (int rep = 0; rep < 2; ++rep) {
    cudaEventRecord(e0, h->st);
    enqueue_nonlinear<R>(h, h->st, z, x, z);
    cudaEventRecord(e1, h->st);
    if (cudaEventSynchronize(e1) != cudaSuccess) return -1.f;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  return best;
}

// RHS0 + nonlinear term + u + dt*du, divided by axz: the assembly of substage k.
template <typename R>
AsmArgs asm_args(const lh_handle* h, int k) {
  AsmArgs a{};
  a.u1 = h->u1; a.u2 = h->u2; a.u3 = h->u3; a.p = h->p;
  a.n1 = h->n1; a.n2 = h->n2; a.n3 = h->n3;
  a.r1 = h->r1; a.r2 = h->r2; a.r3 = h->r3;
  {
    const double2* pr[6] = {h->puu, h->puw, h->pww, h->pvv, h->puv, h->pvw};
    for (int q = 0; q < 6; ++q) {
      if (sizeof(R) == 4) a.p32[q] = reinterpret_cast<const float2*>(pr[q]);
      else a.p64[q] = pr[q];
    }
  }
  a.lytip = h->lytip;
  a.tipu[0] = h->tipu[0]; a.tipu[1] = h->tipu[1]; a.tipv[0] = h->tipv[0]; a.tipv[1] = h->tipv[1];
  a.sc = h->sc;
  a.C1 = h->aRK[k] / h->Re; a.C2 = -h->cRK[k]; a.d = h->dRK[k]; a.g = h->gRK[k];
  a.dt = h->dt; a.beta = h->bRK[k] * h->dt / h->Re; a.k = k;
  return a;
}

// The canopy forcing of substage k: z-inverse of the processed planes, the x pass with the mask, z-forward
// (false without canopy planes).
template <typename R>
bool ib_args(const lh_handle* h, int k, ZJobs<R>* zi, MaskArgs<R>* m, ZJobs<R>* zf) {
  using T2 = cpx_t<R>;
  if (h->nibu + h->nibv == 0) return false;
  const size_t mp = h->d.mp;
  T2* mib = (T2*)h->mixib;
  ZJobs<R> J{};
  J.j[0] = ZJob<R>{h->r1, nullptr, mib, h->ibu_lev, 0, h->nibu};
  J.j[1] = ZJob<R>{h->r3, nullptr, mib + (size_t)h->nibu * mp, h->ibu_lev, 0, h->nibu};
  J.j[2] = ZJob<R>{h->r2, nullptr, mib + (size_t)2 * h->nibu * mp, h->ibv_lev, 0, h->nibv};
  J.j[3] = ZJob<R>{h->lytip, nullptr, (T2*)h->mixly, nullptr, 0, 6};
  J.njobs = 4;
  J.maxlev = std::max(std::max(h->nibu, h->nibv), 6);
  *zi = J;
  MaskArgs<R> a{};
  a.mix = mib;
  a.lymix = (const T2*)h->mixly;
  a.mask[0] = h->ibu_mask; a.mask[1] = h->ibu_mask; a.mask[2] = h->ibv_mask;
  a.tipslot[0] = h->ibu_tip; a.tipslot[1] = h->ibw_tip; a.tipslot[2] = h->ibv_tip;
  a.nplanes[0] = h->nibu; a.nplanes[1] = h->nibu; a.nplanes[2] = h->nibv;
  a.beta = h->bRK[k] * h->dt / h->Re;
  *m = a;
  ZJobs<R> F{};
  F.j[0] = ZJob<R>{nullptr, h->r1, mib, h->ibu_lev, 0, h->nibu};
  F.j[1] = ZJob<R>{nullptr, h->r3, mib + (size_t)h->nibu * mp, h->ibu_lev, 0, h->nibu};
  F.j[2] = ZJob<R>{nullptr, h->r2, mib + (size_t)2 * h->nibu * mp, h->ibv_lev, 0, h->nibv};
  F.njobs = 3;
  F.maxlev = std::max(h->nibu, h->nibv);
  *zf = F;
  return true;
}

// solveP + v_corr of substage k (psolve's scalars)
void psolve_scalars(const lh_handle* h, int k, double* dtirk, double* dtrk) {
  const double dti = 1.0 / h->dt;
  *dtirk = dti / (h->aRK[k] + h->bRK[k]);
  *dtrk = h->dt * (h->aRK[k] + h->bRK[k]);
}

template <typename R>
int enqueue_substage(lh_handle* h, int k, int upto) {
  const Dims& d = h->d;
  cudaStream_t st = h->st;
  enqueue_nonlinear<R>(h, st, true, true, true);
  launch_assemble(asm_args<R>(h, k), d, h->t, st);
  mark(h, K_ASSEMBLE);
  if (upto <= 1) return LH_OK;
  {
    ZJobs<R> zi, zf;
    MaskArgs<R> m;
    if (ib_args<R>(h, k, &zi, &m, &zf)) {
      launch_zinv<R>(zi, d, h->pz.plan, h->tx, st, h->zthreads);
      mark(h, K_IB_ZINV);
      launch_xmask<R>(m, d, h->ph.plan, h->rtw, st);
      mark(h, K_IB_XMASK);
      launch_zfwd<R>(zf, d, h->pz.plan, h->tx, 1.0 / d.ngz, st, h->zthreads);
      mark(h, K_IB_ZFWD);
    }
  }
  if (upto <= 2) return LH_OK;
  launch_vsolve(h->r1, h->r2, h->r3, h->u1, h->u2, h->u3, d, h->t, k, st);
  mark(h, K_VSOLVE);
  if (upto <= 3) return LH_OK;
  if (h->prm.flag_ctpress == 0) {
    launch_flowrate(h->u1, h->sc, d, h->t, k, h->Qx1[k], st);
    mark(h, K_FLOWRATE);
  }
  if (upto <= 4) return LH_OK;
  double dtirk, dtrk;
  psolve_scalars(h, k, &dtirk, &dtrk);
  launch_psolve(h->u1, h->u2, h->u3, h->p, h->psi, d, h->t, dtirk, dtrk, h->gw[0][0], h->gw[2][1], h->sc, st);
  mark(h, K_PSOLVE);
  return LH_OK;
}

int substage(lh_handle* h, int k, int upto) {
  int rc = h->precision == LH_PREC_MIXED ? enqueue_substage<float>(h, k, upto) : enqueue_substage<double>(h, k, upto);
  if (rc) return rc;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(h, LH_ECUDA, "kernel launch: %s", cudaGetErrorString(e));
  return LH_OK;
}

int count_launches(const lh_handle* h) {
  // zinv, xprod, zfwd per band; assemble, vsolve, psolve (+flowrate)
  int per = 3 * (h->d.banded ? 3 : 1) + 3 + (h->prm.flag_ctpress == 0 ? 1 : 0);
  if (h->nibu + h->nibv > 0) per += 3;
  return 3 * per;
}

void free_all(lh_handle* h) {
  if (h->graph) cudaGraphExecDestroy(h->graph);
  for (void* p : h->allocs) cudaFree(p);
  h->allocs.clear();
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->own_stream && h->st) cudaStreamDestroy(h->st);
}

// Host field (either layout) -> device planes
int put_field(lh_handle* h, double2* dst, const double* src, char grid, int layout) {
  const size_t n = field_elems(h, grid);
  if (layout == LH_LAYOUT_PLANES) {
    CU(h, cudaMemcpyAsync(dst, src, n * sizeof(double2), cudaMemcpyHostToDevice, h->st));
  } else if (layout == LH_LAYOUT_COLUMNS) {
    const int ny = (int)(n / h->d.np);
    CU(h, cudaMemcpyAsync(h->stage, src, n * sizeof(double2), cudaMemcpyHostToDevice, h->st));
    launch_transpose(h->stage, dst, h->d.np, ny, h->st);  // [col][j] -> [j][col]
  } else {
    return fail(h, LH_EINVAL, "unknown layout %d", layout);
  }
  CU(h, cudaStreamSynchronize(h->st));
  return LH_OK;
}

int get_field(lh_handle* h, double* dst, const double2* src, char grid, int layout) {
  const size_t n = field_elems(h, grid);
  if (layout == LH_LAYOUT_PLANES) {
    CU(h, cudaMemcpyAsync(dst, src, n * sizeof(double2), cudaMemcpyDeviceToHost, h->st));
  } else if (layout == LH_LAYOUT_COLUMNS) {
    const int ny = (int)(n / h->d.np);
    launch_transpose(src, h->stage, ny, h->d.np, h->st);  // [j][col] -> [col][j]
    CU(h, cudaMemcpyAsync(dst, h->stage, n * sizeof(double2), cudaMemcpyDeviceToHost, h->st));
  } else {
    return fail(h, LH_EINVAL, "unknown layout %d", layout);
  }
  CU(h, cudaStreamSynchronize(h->st));
  return LH_OK;
}

int read_scalars(lh_handle* h, DevScalars* out) {
  CU(h, cudaMemcpyAsync(out, h->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->st));
  CU(h, cudaStreamSynchronize(h->st));
  return LH_OK;
}

// flowrateIm of the current (0,0) column, on the host
int host_flowrate(lh_handle* h, double* Q) {
  const Dims& d = h->d;
  std::vector<double2> col(d.nn + 2);
  // the (0,0) mode of levels 0..nn+1, gathered on the device into scratch and read back in one copy
  launch_gather_col(h->u1 + (size_t)(0 - d.ju0) * d.np, d.np, d.nn + 2, h->stage, h->st);
  CU(h, cudaMemcpyAsync(col.data(), h->stage, sizeof(double2) * (d.nn + 2), cudaMemcpyDeviceToHost, h->st));
  CU(h, cudaStreamSynchronize(h->st));
  double q = 0.0;
  for (int j = 1; j <= d.nn + 1; ++j) q = q + (h->yv[j - d.ju0] - h->yv[j - 1 - d.ju0]) * col[j].x;
  *Q = q;
  return LH_OK;
}

// The sticky error bits of the device scalars (read after the stream has finished).
int read_err(lh_handle* h, int* err) {
  CU(h, cudaMemcpyAsync(err, &h->sc->err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CU(h, cudaStreamSynchronize(h->st));
  return LH_OK;
}

// error (littleharsh.f90:323-352): max |div u| over the p grid, on the device.
int device_divmax(lh_handle* h, double* out) {
  CU(h, cudaMemsetAsync(&h->sc->cflbits, 0, sizeof(unsigned long long), h->st));
  launch_divergence(h->u1, h->u2, h->u3, h->psi, h->d, h->t, h->st);
  launch_absmax(h->psi, field_elems(h, 'p'), h->sc, h->st);
  DevScalars s;
  int rc = read_scalars(h, &s);
  if (rc) return rc;
  unsigned long long b = s.cflbits;
  std::memcpy(out, &b, sizeof(double));
  CU(h, cudaGetLastError());
  return LH_OK;
}

}  // namespace

namespace lh {
int make_dims(const lh_params* prm, Dims* out, std::string* why) {
  auto Nf = [&](int row, int band) { return prm->N[band * 4 + row - 1]; };
  auto Gf = [&](int row, int band) { return prm->Ngal[band * 4 + row - 1]; };
  auto no = [&](int code, const char* msg) {
    *why = msg;
    return code;
  };
  Dims d{};
  d.ngx = Gf(1, 1); d.ngz = Gf(2, 1);
  const int nx = Nf(1, 1), nz = Nf(2, 1);
  if (nx != 2 * (d.ngx / 3) || nz != 2 * (d.ngz / 3) || d.ngx < 6 || d.ngz < 6 || (d.ngx & 1) || (nz & 1))
    return no(LH_EINVAL, "inconsistent N/Ngal");
  d.nkx = nx / 2 + 1;
  d.nz = nz;
  d.np = d.nkx * d.nz;
  d.mp = d.nkx * d.ngz;
  d.spitch = d.nkx;
  d.snz = d.nz;
  d.ju0 = Nf(4, 0);
  // variable-resolution bands (start.f90:95-118): the middle band's resolution
  d.ngx2 = Gf(1, 2); d.ngz2 = Gf(2, 2);
  d.banded = (d.ngx2 != d.ngx || d.ngz2 != d.ngz);
  {
    const int nx2 = Nf(1, 2), nz2 = Nf(2, 2);
    if (nx2 != 2 * (d.ngx2 / 3) || nz2 != 2 * (d.ngz2 / 3) || d.ngx2 < 6 || d.ngz2 < 6 || (d.ngx2 & 1) || (nz2 & 1) ||
        d.ngx2 > d.ngx || d.ngz2 > d.ngz || Gf(1, 3) != d.ngx || Gf(2, 3) != d.ngz)
      return no(LH_EINVAL, "inconsistent band resolutions (the middle band may not be finer than the walls')");
    d.nkx2 = nx2 / 2 + 1;
    d.nz2 = nz2;
  }
  d.Nu1 = Nf(4, 1) - d.ju0; d.Nu2 = Nf(4, 2) - d.ju0;
  d.Nv1 = Nf(3, 1) - d.ju0; d.Nv2 = Nf(3, 2) - d.ju0;
  if (Nf(3, 0) != d.ju0) return no(LH_EINVAL, "N(3,0) != N(4,0)");
  d.nyu = Nf(4, 3) + 1 - Nf(4, 0) + 1;
  d.nyv = Nf(3, 3) + 1 - Nf(3, 0) + 1;
  d.nyp = Nf(4, 3) - (Nf(4, 0) + 1) + 1;
  d.nn = prm->nn;
  if (d.nyv != d.nyu - 1 || d.nyp != d.nyu - 2 || d.nyu < 6) return no(LH_EINVAL, "inconsistent y grid sizes");
  if (d.nn + 2 - d.ju0 >= d.nyu || d.ju0 > 0) return no(LH_EINVAL, "nn outside the u grid");
  if (d.banded && !(d.Nu1 >= 2 && d.Nv1 == d.Nu1 - 1 && d.Nu2 > d.Nu1 + 1 && d.Nv2 == d.Nu2 && d.Nu2 < d.nyu - 3))
    return no(LH_EINVAL, "band limits N(3:4,1:2) do not describe three bands");
  if (!(prm->Re > 0) || !(prm->alp > 0) || !(prm->bet > 0)) return no(LH_EINVAL, "Re, alp, bet must be positive");
  *out = d;
  return LH_OK;
}

void set_init_error(const char* msg) { g_init_error = msg; }
void set_handle_error(lh_handle* h, const char* msg) {
  if (h) h->err = msg;
  else g_init_error = msg;
}
}  // namespace lh

extern "C" {

const char* lh_last_error(const lh_handle* h) { return h ? h->err.c_str() : g_init_error.c_str(); }

int lh_init(const lh_params* prm, const double* yu, const double* yv, const double* dthdyu, const double* dthdyv,
            const double* dyu2i, const double* dyv2i, const int32_t* list_u, int32_t nlist_u, const int32_t* list_v,
            int32_t nlist_v, lh_handle** out) {
  if (!out) return fail(nullptr, LH_EINVAL, "out is NULL");
  *out = nullptr;
  if (!prm || !yu || !yv || !dthdyu || !dthdyv || !dyu2i || !dyv2i) return fail(nullptr, LH_EINVAL, "NULL argument");
  if (prm->abi_version != LH_ABI_VERSION) return fail(nullptr, LH_EINVAL, "abi_version %d != %d", prm->abi_version, LH_ABI_VERSION);
  auto Nf = [&](int row, int band) { return prm->N[band * 4 + row - 1]; };
  auto Gf = [&](int row, int band) { return prm->Ngal[band * 4 + row - 1]; };
  if (prm->precision != LH_PREC_FP64 && prm->precision != LH_PREC_MIXED) return fail(nullptr, LH_EINVAL, "bad precision");
  if (prm->geometry_type != 0 && prm->geometry_type != 3) return fail(nullptr, LH_EUNSUPPORTED, "geometry_type %d has no forcing builder", prm->geometry_type);
  Dims dims{};
  {  // the parameter block is checked before any CUDA call
    std::string why;
    const int rc = make_dims(prm, &dims, &why);
    if (rc) return fail(nullptr, rc, "%s", why.c_str());
  }
  lh_handle* h = new lh_handle();
  h->prm = *prm;
  h->precision = prm->precision;
  cudaGetDevice(&h->device);
  if (prm->stream) {
    h->st = static_cast<cudaStream_t>(prm->stream);
  } else {
    if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) {
      delete h;
      return fail(nullptr, LH_ECUDA, "cannot create a stream (is a CUDA device available?)");
    }
    h->own_stream = true;
  }
  auto bail = [&](int rc) {
    g_init_error = h->err;
    free_all(h);
    delete h;
    return rc;
  };
  Dims& d = h->d;
  d = dims;
  const int nx = Nf(1, 1), nz = Nf(2, 1);
  h->Re = prm->Re; h->alp = prm->alp; h->bet = prm->bet;
  h->Lx = 2.0 * (double)kPi / h->alp;
  h->Lz = 2.0 * (double)kPi / h->bet;
  for (int c = 0; c < 2; ++c)
    for (int b = 0; b < 3; ++b) h->gw[b][c] = prm->gridweighting[c * 3 + b];
  h->yu.assign(yu, yu + d.nyu);
  h->yv.assign(yv, yv + d.nyv);
  h->dthdyu.assign(dthdyu, dthdyu + d.nyu);
  h->dthdyv.assign(dthdyv, dthdyv + d.nyv);
  h->dyu2i.assign(dyu2i, dyu2i + 3 * d.nyu);
  h->dyv2i.assign(dyv2i, dyv2i + 3 * d.nyv);
  // def_k (start.f90:655-704)
  h->kx.resize(d.nkx); h->k2x.resize(d.nkx); h->kz.resize(nz); h->k2z.resize(nz);
  for (int i = 0; i < d.nkx; ++i) { h->kx[i] = h->alp * i; h->k2x[i] = -((h->alp * i) * (h->alp * i)); }
  for (int k = 1; k <= nz; ++k) {
    const double a = k <= nz / 2 ? h->bet * (k - 1) : h->bet * (nz - k + 1);
    h->kz[k - 1] = k <= nz / 2 ? a : -a;
    h->k2z[k - 1] = -(a * a);
  }
  // RK3 (start.f90:413-427)
  const double aR[3] = {4.0 / 15.0, 1.0 / 15.0, 1.0 / 6.0}, gR[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
  const double cR[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0}, dR[3] = {8.0 / 15.0, 2.0 / 15.0, 1.0 / 3.0};
  for (int k = 0; k < 3; ++k) { h->aRK[k] = aR[k]; h->bRK[k] = aR[k]; h->gRK[k] = gR[k]; h->cRK[k] = cR[k]; h->dRK[k] = dR[k]; }
  {
    const double dyw = h->yv[1] - h->yv[0];
    h->dtv = h->Re / (-h->k2x[nx / 2] - h->k2z[nz / 2 - 1] + 4.0 / (dyw * dyw));
  }
  int rc;
  // FFT plans: z of length ngz, x through a complex transform of ngx/2
  if ((rc = build_plan(h, h->pz, d.ngz, d.nz / 2)) || (rc = build_plan(h, h->ph, d.ngx / 2, 0)) ||
      (rc = build_plan(h, h->pf, d.ngx, 0)))
    return bail(rc);
  if (d.banded) {
    // the middle band's planes: their own transform lengths and mode counts, the same storage
    Dims& c = h->dmid;
    c = d;
    c.ngx = d.ngx2; c.ngz = d.ngz2; c.nkx = d.nkx2; c.nz = d.nz2;
    c.mp = c.nkx * c.ngz;
    if ((rc = build_plan(h, h->pz2, c.ngz, c.nz / 2)) || (rc = build_plan(h, h->ph2, c.ngx / 2, 0)) ||
        (rc = build_plan(h, h->pf2, c.ngx, 0)))
      return bail(rc);
    std::vector<double2> rt(c.ngx / 2 + 1);
    for (int k = 0; k <= c.ngx / 2; ++k) {
      const long double a = 2.0L * kPi * (long double)k / (long double)c.ngx;
      rt[k] = double2{(double)cosl(a), -(double)sinl(a)};
    }
    if ((rc = upload(h, &h->rtw2, rt))) return bail(rc);
  }
  {
    std::vector<double2> rt(d.ngx / 2 + 1);
    for (int k = 0; k <= d.ngx / 2; ++k) {
      const long double a = 2.0L * kPi * (long double)k / (long double)d.ngx;
      rt[k] = double2{(double)cosl(a), -(double)sinl(a)};
    }
    if ((rc = upload(h, &h->rtw, rt))) return bail(rc);
  }
  // small tables
  {
    std::vector<double> cu(d.nyu), cv(d.nyv), wc(d.nyu, 0.0), wf(d.nyv, 0.0), dyc(d.nyu, 0.0), dyvw(d.nn + 2, 0.0);
    for (int j = 0; j < d.nyu; ++j) cu[j] = prm->ddthetavi * h->dthdyu[j];
    for (int j = 0; j < d.nyv; ++j) cv[j] = prm->ddthetavi * h->dthdyv[j];
    for (int j = 1; j < d.nyu - 1; ++j) {
      wc[j] = (h->yu[j] - h->yv[j - 1]) / (h->yv[j] - h->yv[j - 1]);
      dyc[j] = 1.0 / (h->yv[j] - h->yv[j - 1]);
    }
    for (int j = 1; j < d.nyv - 1; ++j) wf[j] = (h->yv[j] - h->yu[j]) / (h->yu[j + 1] - h->yu[j]);
    for (int j = 1; j <= d.nn + 1; ++j) dyvw[j] = h->yv[j - d.ju0] - h->yv[j - 1 - d.ju0];
    double *pkx, *pkz, *pk2x, *pk2z, *pd2u, *pd2v, *pcu, *pcv, *pwc, *pwf, *pdyc, *pdyvw;
    if ((rc = upload(h, &pkx, h->kx)) || (rc = upload(h, &pkz, h->kz)) || (rc = upload(h, &pk2x, h->k2x)) ||
        (rc = upload(h, &pk2z, h->k2z)) || (rc = upload(h, &pd2u, h->dyu2i)) || (rc = upload(h, &pd2v, h->dyv2i)) ||
        (rc = upload(h, &pcu, cu)) || (rc = upload(h, &pcv, cv)) || (rc = upload(h, &pwc, wc)) ||
        (rc = upload(h, &pwf, wf)) || (rc = upload(h, &pdyc, dyc)) || (rc = upload(h, &pdyvw, dyvw)))
      return bail(rc);
    h->t.kx = pkx; h->t.kz = pkz; h->t.k2x = pk2x; h->t.k2z = pk2z; h->t.d2u = pd2u; h->t.d2v = pd2v;
    h->t.cu = pcu; h->t.cv = pcv; h->t.wc = pwc; h->t.wf = pwf; h->t.dyc = pdyc; h->t.dyvw = pdyvw;
    // the same values rounded to float (to nearest, as a device conversion would round them)
    auto rounded = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
    float *pkxf, *pkzf, *pcuf, *pcvf;
    if ((rc = upload(h, &pkxf, rounded(h->kx))) || (rc = upload(h, &pkzf, rounded(h->kz))) ||
        (rc = upload(h, &pcuf, rounded(cu))) || (rc = upload(h, &pcvf, rounded(cv))))
      return bail(rc);
    h->t.kxf = pkxf; h->t.kzf = pkzf; h->t.cuf = pcuf; h->t.cvf = pcvf;
  }
  // pressure LU per column (LU_buildP + LU_decP)
  {
    const int np_ = d.nyp;
    std::vector<double> rows(4 * (size_t)np_), dg1(np_);
    const double dv = prm->ddthetavi;
    for (int jp = 0; jp < np_; ++jp) {
      const int ju = jp + 1, jvv = jp + 1;  // centre j on the u grid, face j on the v grid
      const double Dt = dv * h->dthdyu[ju], Dbm = -dv * h->dthdyu[ju];          // D_t(j), D_b(j-1)
      const double Gb = -dv * h->dthdyv[jvv], Gtp = dv * h->dthdyv[jvv];        // G_b(j), G_t(j+1)
      const double Gt = jp > 0 ? dv * h->dthdyv[jvv - 1] : 0.0;                 // G_t(j) = ddthetavi*dthdyv(j-1)
      const double Gbm = jp > 0 ? -dv * h->dthdyv[jvv - 1] : 0.0;               // G_b(j-1)
      rows[4 * jp + 0] = Dbm * Gt;
      rows[4 * jp + 1] = Dt * Gb;
      rows[4 * jp + 2] = Dbm * Gbm;
      rows[4 * jp + 3] = Dt * Gtp;
      dg1[jp] = rows[4 * jp + 2];
    }
    double *prows, *pdg1, *pdg2, *pdg3;
    if ((rc = upload(h, &prows, rows)) || (rc = upload(h, &pdg1, dg1)) ||
        (rc = dalloc(h, &pdg2, (size_t)np_ * d.np)) || (rc = dalloc(h, &pdg3, (size_t)np_ * d.np)))
      return bail(rc);
    // the (0,0) Dirichlet row uses yu at global indices 1 and 2 (tridLU_3D_IB.f90:551)
    const double dy12 = h->yu[2 - d.ju0] - h->yu[1 - d.ju0];
    const double pin = 1.0 / (dy12 * dy12);
    h->t.dg1 = pdg1; h->t.dg2 = pdg2; h->t.dg3 = pdg3;
    launch_build_dg(pdg2, pdg3, prows, d, h->t, pin, h->st);
  }
  // canopy forcing planes and masks (getbounds filtering, start.f90:780-990)
  {
    const int dsty = prm->dsty;
    const int ngal43 = Gf(4, 3), ngal33 = Gf(3, 3);
    std::vector<int> levu, levv;
    if (prm->geometry_type == 3) {
      const int ulo = Nf(4, 0) + 1, uhi = Nf(4, 3), vlo = Nf(3, 0) + 1, vhi = Nf(3, 3);
      const int ur[2][2] = {{-dsty + 1, 0}, {ngal43 - dsty + 1, ngal43}};
      const int vr[2][2] = {{-dsty, -1}, {ngal33 + 1 - dsty + 1, ngal33 + 1}};
      for (int c = 0; c < 2; ++c) {
        for (int j = std::max(ur[c][0], ulo); j <= std::min(ur[c][1], uhi); ++j) levu.push_back(j - d.ju0);
        for (int j = std::max(vr[c][0], vlo); j <= std::min(vr[c][1], vhi); ++j) levv.push_back(j - d.ju0);
      }
      h->tipu[0] = 0 - d.ju0; h->tipu[1] = ngal43 - dsty + 1 - d.ju0;
      h->tipv[0] = -1 - d.ju0; h->tipv[1] = ngal33 - dsty + 2 - d.ju0;
    }
    h->nibu = (int)levu.size();
    h->nibv = (int)levv.size();
    for (int l : levu)
      if (coarse_u(d, l)) return bail(fail(h, LH_EUNSUPPORTED, "canopy planes must lie in the wall bands"));
    for (int l : levv)
      if (coarse_v(d, l)) return bail(fail(h, LH_EUNSUPPORTED, "canopy planes must lie in the wall bands"));
    const size_t pl = (size_t)d.ngx * d.ngz;
    std::vector<uint8_t> mu(pl * std::max(h->nibu, 1), 0), mv(pl * std::max(h->nibv, 1), 0);
    auto mark = [&](const int32_t* L, int n, const std::vector<int>& lev, std::vector<uint8_t>& m) -> int {
      for (int q = 0; q < n; ++q) {
        const int i = L[3 * q], k = L[3 * q + 1], j = L[3 * q + 2];
        int slot = -1;
        for (size_t s = 0; s < lev.size(); ++s)
          if (lev[s] == j - d.ju0) { slot = (int)s; break; }
        if (slot < 0) continue;  // outside the processed planes: dropped, as getbounds does
        if (i < 1 || i > d.ngx || k < 1 || k > d.ngz) return -1;
        m[(size_t)slot * pl + (size_t)(k - 1) * d.ngx + (i - 1)] = 1;
      }
      return 0;
    };
    if (h->nibu && (!list_u || nlist_u < 0)) return bail(fail(h, LH_EINVAL, "canopy list for the u grid missing"));
    if (h->nibv && (!list_v || nlist_v < 0)) return bail(fail(h, LH_EINVAL, "canopy list for the v grid missing"));
    if (h->nibu && mark(list_u, nlist_u, levu, mu)) return bail(fail(h, LH_EINVAL, "canopy point outside the plane"));
    if (h->nibv && mark(list_v, nlist_v, levv, mv)) return bail(fail(h, LH_EINVAL, "canopy point outside the plane"));
    std::vector<int> tu(std::max(h->nibu, 1), -1), tw(std::max(h->nibu, 1), -1), tv(std::max(h->nibv, 1), -1);
    for (int s = 0; s < h->nibu; ++s) {
      if (levu[s] == h->tipu[0]) { tu[s] = 0; tw[s] = 2; }
      if (levu[s] == h->tipu[1]) { tu[s] = 1; tw[s] = 3; }
    }
    for (int s = 0; s < h->nibv; ++s) {
      if (levv[s] == h->tipv[0]) tv[s] = 4;
      if (levv[s] == h->tipv[1]) tv[s] = 5;
    }
    if (levu.empty()) levu.push_back(0);
    if (levv.empty()) levv.push_back(0);
    if ((rc = upload(h, &h->ibu_lev, levu)) || (rc = upload(h, &h->ibv_lev, levv)) || (rc = upload(h, &h->ibu_mask, mu)) ||
        (rc = upload(h, &h->ibv_mask, mv)) || (rc = upload(h, &h->ibu_tip, tu)) || (rc = upload(h, &h->ibw_tip, tw)) ||
        (rc = upload(h, &h->ibv_tip, tv)))
      return bail(rc);
  }
  // fields and scratch
  {
    const size_t fu = field_elems(h, 'u'), fv = field_elems(h, 'v'), fp = field_elems(h, 'p');
    if ((rc = dalloc(h, &h->u1, fu)) || (rc = dalloc(h, &h->u3, fu)) || (rc = dalloc(h, &h->u2, fv)) ||
        (rc = dalloc(h, &h->p, fp)) || (rc = dalloc(h, &h->n1, fu)) || (rc = dalloc(h, &h->n3, fu)) ||
        (rc = dalloc(h, &h->n2, fv)) || (rc = dalloc(h, &h->r1, fu)) || (rc = dalloc(h, &h->r3, fu)) ||
        (rc = dalloc(h, &h->r2, fv)) || (rc = dalloc(h, &h->puu, fu)) || (rc = dalloc(h, &h->puw, fu)) ||
        (rc = dalloc(h, &h->pww, fu)) || (rc = dalloc(h, &h->pvv, fu)) || (rc = dalloc(h, &h->puv, fv)) ||
        (rc = dalloc(h, &h->pvw, fv)) || (rc = dalloc(h, &h->psi, fp)) || (rc = dalloc(h, &h->stage, fu)) ||
        (rc = dalloc(h, &h->lytip, 6 * (size_t)d.np)) || (rc = dalloc(h, &h->sc, 1)))
      return bail(rc);
    const size_t cb = h->precision == LH_PREC_MIXED ? sizeof(float2) : sizeof(double2);
    const size_t mu = (size_t)d.nyu * d.mp, mv = (size_t)d.nyv * d.mp;
    unsigned char* m;
    // mixu, mixw (u grid), mixv (v grid), then products uu, uw, ww, vv (u grid) and uv, vw (v grid)
    if ((rc = dalloc(h, &m, cb * (6 * mu + 3 * mv)))) return bail(rc);
    h->mixu = m; m += cb * mu;
    h->mixw = m; m += cb * mu;
    h->mixv = m; m += cb * mv;
    for (int i = 0; i < 6; ++i) { h->mixp[i] = m; m += cb * (i < 4 ? mu : mv); }
    const size_t nib = 2 * (size_t)h->nibu + h->nibv;
    if ((rc = dalloc(h, &m, cb * (size_t)d.mp * (nib + 6)))) return bail(rc);
    h->mixib = m;
    h->mixly = m + cb * (size_t)d.mp * nib;
    if ((rc = dalloc(h, &h->spec, (3 * (size_t)d.nyu + d.nyv + d.nyp) * d.np))) return bail(rc);
    if ((rc = dalloc(h, &h->stat, 13 * (size_t)std::max(d.nyu, d.nyv)))) return bail(rc);
    if (prm->geometry_type == 3) {
      if (prm->ntilex <= 0 || prm->ntilez <= 0 || d.ngx % prm->ntilex || d.ngz % prm->ntilez)
        return bail(fail(h, LH_EINVAL, "ntilex/ntilez must be positive and divide Ngalx/Ngalz"));
      h->dnx = d.ngx / prm->ntilex;
      h->dnz = d.ngz / prm->ntilez;
      h->nju = Nf(4, 1) - Nf(4, 0) + 1;
      h->njv = Nf(3, 1) - Nf(3, 0) + 1;
      h->njp = Nf(4, 1) - Nf(4, 0) - 1;
      if (h->nju < 1 || h->njv < 1 || h->njp < 1 || 2 * h->nju > d.nyu || 2 * h->njv > d.nyv || 2 * h->njp > d.nyp)
        return bail(fail(h, LH_EINVAL, "wall bands inconsistent with the y grid"));
      std::vector<int> ul(2 * h->nju), vl(2 * h->njv), pl(2 * h->njp);
      for (int j = 0; j < h->nju; ++j) { ul[2 * j] = j; ul[2 * j + 1] = d.nyu - 1 - j; }
      for (int j = 0; j < h->njv; ++j) { vl[2 * j] = j; vl[2 * j + 1] = d.nyv - 1 - j; }
      for (int j = 0; j < h->njp; ++j) { pl[2 * j] = j; pl[2 * j + 1] = d.nyp - 1 - j; }
      const size_t tile = (size_t)h->dnx * h->dnz;
      if ((rc = upload(h, &h->cond_ul, ul)) || (rc = upload(h, &h->cond_vl, vl)) || (rc = upload(h, &h->cond_pl, pl)) ||
          (rc = dalloc(h, &h->cond, tile * (6 * (size_t)h->nju + 5 * (size_t)h->njv + 2 * (size_t)h->njp))))
        return bail(rc);
    }
  }
  // launch shapes: z tile width and levels per x-pass chunk
  // z tile width: narrow tiles keep several CTAs per SM so that one CTA's loads overlap another's
  // butterflies (measured on configuration 2: FP64 best at 4, mixed at 8)
  h->tx = h->precision == LH_PREC_MIXED ? 8 : 4;
  h->chunk = d.nyu > 256 ? 32 : 16;
  // launch-shape overrides for tuning sweeps: LH_TX (z tile width, 1..64), LH_CHUNK (levels per x-pass CTA)
  if (const char* v = std::getenv("LH_TX")) { const int x = std::atoi(v); if (x >= 1 && x <= 64) h->tx = x; }
  if (const char* v = std::getenv("LH_CHUNK")) { const int x = std::atoi(v); if (x >= 1 && x <= 4096) h->chunk = x; }
  if (const char* v = std::getenv("LH_XSPLIT")) h->xsplit = std::atoi(v) != 0 ? 1 : 0;
  if (const char* v = std::getenv("LH_XTHREADS")) h->xthreads = std::atoi(v) == 128 ? 128 : 256;
  if (const char* v = std::getenv("LH_ZTHREADS")) h->zthreads = std::atoi(v) == 128 ? 128 : 256;
  if (const char* v = std::getenv("LH_XROWS")) h->xrows = std::atoi(v) == 2 ? 2 : 1;
  {
    const cudaError_t e = configure_kernels();
    if (e != cudaSuccess) return bail(fail(h, LH_ECUDA, "kernel attributes: %s", cudaGetErrorString(e)));
  }
  if (cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)
    return bail(fail(h, LH_ECUDA, "cudaEventCreate failed"));
  {
    DevScalars s{};
    if (cudaMemcpyAsync(h->sc, &s, sizeof s, cudaMemcpyHostToDevice, h->st) != cudaSuccess)
      return bail(fail(h, LH_ECUDA, "scalar upload failed"));
  }
  if (cudaStreamSynchronize(h->st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return bail(fail(h, LH_ECUDA, "set-up kernels failed: %s", cudaGetErrorString(cudaGetLastError())));
  h->launches_per_step = count_launches(h);
  *out = h;
  return LH_OK;
}

void lh_free(lh_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->st) cudaStreamSynchronize(h->st);
  free_all(h);
  delete h;
}

int lh_get_sizes(const lh_handle* h, int32_t* o) {
  if (!h || !o) return LH_EINVAL;
  const Dims& d = h->d;
  const int v[12] = {d.nkx, d.nz, d.ngx, d.ngz, d.nyu, d.nyv, d.nyp, d.ju0, d.ju0, d.ju0 + 1, h->nibu, h->nibv};
  std::memcpy(o, v, sizeof v);
  return LH_OK;
}

int lh_set_fields(lh_handle* h, const double* u1, const double* u2, const double* u3, const double* p, int32_t layout) {
  if (!h) return LH_EINVAL;
  cudaSetDevice(h->device);
  int rc;
  if (u1 && (rc = put_field(h, h->u1, u1, 'u', layout))) return rc;
  if (u2 && (rc = put_field(h, h->u2, u2, 'v', layout))) return rc;
  if (u3 && (rc = put_field(h, h->u3, u3, 'u', layout))) return rc;
  if (p && (rc = put_field(h, h->p, p, 'p', layout))) return rc;
  if (u1 && h->prm.flag_ctpress != 1) {
    double Q;
    if ((rc = host_flowrate(h, &Q))) return rc;
    CU(h, cudaMemcpyAsync(&h->sc->QxT, &Q, sizeof Q, cudaMemcpyHostToDevice, h->st));
  }
  // new fields: the sticky error bits of the old ones no longer apply
  CU(h, cudaMemsetAsync(&h->sc->err, 0, sizeof(int), h->st));
  CU(h, cudaStreamSynchronize(h->st));
  h->have_fields = true;
  return LH_OK;
}

int lh_get_fields(lh_handle* h, double* u1, double* u2, double* u3, double* p, int32_t layout) {
  if (!h) return LH_EINVAL;
  cudaSetDevice(h->device);
  int rc;
  if (u1 && (rc = get_field(h, u1, h->u1, 'u', layout))) return rc;
  if (u2 && (rc = get_field(h, u2, h->u2, 'v', layout))) return rc;
  if (u3 && (rc = get_field(h, u3, h->u3, 'u', layout))) return rc;
  if (p && (rc = get_field(h, p, h->p, 'p', layout))) return rc;
  return LH_OK;
}

int lh_set_nonlinear(lh_handle* h, const double* n1, const double* n2, const double* n3, int32_t layout) {
  if (!h) return LH_EINVAL;
  cudaSetDevice(h->device);
  int rc;
  if (n1 && (rc = put_field(h, h->n1, n1, 'u', layout))) return rc;
  if (n2 && (rc = put_field(h, h->n2, n2, 'v', layout))) return rc;
  if (n3 && (rc = put_field(h, h->n3, n3, 'u', layout))) return rc;
  return LH_OK;
}

int lh_get_nonlinear(lh_handle* h, double* n1, double* n2, double* n3, int32_t layout) {
  if (!h) return LH_EINVAL;
  cudaSetDevice(h->device);
  int rc;
  if (n1 && (rc = get_field(h, n1, h->n1, 'u', layout))) return rc;
  if (n2 && (rc = get_field(h, n2, h->n2, 'v', layout))) return rc;
  if (n3 && (rc = get_field(h, n3, h->n3, 'u', layout))) return rc;
  return LH_OK;
}

int lh_get_rhs(lh_handle* h, double* r1, double* r2, double* r3, int32_t layout) {
  if (!h) return LH_EINVAL;
  cudaSetDevice(h->device);
  int rc;
  if (r1 && (rc = get_field(h, r1, h->r1, 'u', layout))) return rc;
  if (r2 && (rc = get_field(h, r2, h->r2, 'v', layout))) return rc;
  if (r3 && (rc = get_field(h, r3, h->r3, 'u', layout))) return rc;
  return LH_OK;
}

int lh_set_time(lh_handle* h, double t, double dt, double mpgx, double QxT) {
  if (!h) return LH_EINVAL;
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(h, LH_EINVAL, "dt must be positive and finite");
  cudaSetDevice(h->device);
  h->t_now = t;
  if (dt != h->dt || !h->have_dt) {
    h->dt = dt;
    h->have_dt = true;
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    ++h->graph_gen;
    int rc = build_dt_tables(h);
    if (rc) return rc;
  }
  CU(h, cudaMemcpyAsync(&h->sc->mpgx, &mpgx, sizeof mpgx, cudaMemcpyHostToDevice, h->st));
  if (QxT >= 0.0) CU(h, cudaMemcpyAsync(&h->sc->QxT, &QxT, sizeof QxT, cudaMemcpyHostToDevice, h->st));
  CU(h, cudaStreamSynchronize(h->st));
  return LH_OK;
}

int lh_get_time(lh_handle* h, double* o) {
  if (!h || !o) return LH_EINVAL;
  cudaSetDevice(h->device);
  DevScalars s;
  int rc = read_scalars(h, &s);
  if (rc) return rc;
  double Q;
  if ((rc = host_flowrate(h, &Q))) return rc;
  o[0] = h->t_now; o[1] = h->dt; o[2] = s.mpgx; o[3] = s.QxT; o[4] = Q;
  return LH_OK;
}

int lh_substage(lh_handle* h, int32_t krk, int32_t upto) {
  if (!h) return LH_EINVAL;
  if (krk < 1 || krk > 3) return fail(h, LH_EINVAL, "kRK must be 1..3");
  if (!h->have_fields || !h->have_dt) return fail(h, LH_ESTATE, "fields and dt must be set first");
  cudaSetDevice(h->device);
  int rc = substage(h, krk - 1, upto);
  if (rc) return rc;
  CU(h, cudaStreamSynchronize(h->st));
  return LH_OK;
}

int lh_rk3_step(lh_handle* h, int32_t nsteps) {
  if (!h) return LH_EINVAL;
  if (nsteps < 0) return fail(h, LH_EINVAL, "nsteps < 0");
  if (!h->have_fields || !h->have_dt) return fail(h, LH_ESTATE, "fields and dt must be set first");
  cudaSetDevice(h->device);
  if (!h->graph) {
    cudaGraph_t g = nullptr;
    CU(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    int rc = LH_OK;
    for (int k = 0; k < 3 && rc == LH_OK; ++k) rc = substage(h, k, 5);
    cudaError_t e = cudaStreamEndCapture(h->st, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return fail(h, LH_ECUDA, "graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { h->graph = nullptr; return fail(h, LH_ECUDA, "graph instantiate: %s", cudaGetErrorString(e)); }
  }
  // steps run in blocks of mon_every (all at once without the monitor); after each block the sticky
  // non-finite flag of the pressure solve is read, and with the monitor max |div| is checked against maxerr
  double total_ms = 0.0;
  for (int done = 0; done < nsteps;) {
    const int n = h->mon_every > 0 ? std::min(h->mon_every, nsteps - done) : nsteps - done;
    CU(h, cudaEventRecord(h->ev0, h->st));
    for (int q = 0; q < n; ++q) CU(h, cudaGraphLaunch(h->graph, h->st));
    CU(h, cudaEventRecord(h->ev1, h->st));
    CU(h, cudaEventSynchronize(h->ev1));
    float ms = 0.f;
    CU(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    total_ms += ms;
    done += n;
    h->t_now += n * h->dt;
    h->iter += n;
    h->last_ms = total_ms;
    int err = 0;
    int rc = read_err(h, &err);
    if (rc) return rc;
    if (err & kErrNonFinite)
      return fail(h, LH_ENUMERIC, "non-finite value in the fields within steps %lld..%lld", h->iter - n + 1, h->iter);
    if (h->mon_every > 0) {
      double dm = 0.0;
      if ((rc = device_divmax(h, &dm))) return rc;
      h->last_divmax = dm;
      if (!(dm <= h->mon_maxerr))
        return fail(h, LH_ENUMERIC, "max |div| %.3e exceeds maxerr %.3e after step %lld", dm, h->mon_maxerr, h->iter);
    }
  }
  if (nsteps == 0) h->last_ms = 0.0;
  return LH_OK;
}

int lh_fp64_peak(double* tflops) {
  if (!tflops) return LH_EINVAL;
  const double tf = fp64_probe_tflops(nullptr);
  if (!(tf > 0.0)) return fail(nullptr, LH_ECUDA, "FP64 probe failed");
  *tflops = tf;
  return LH_OK;
}

int lh_set_monitor(lh_handle* h, double maxerr, int32_t every) {
  if (!h) return LH_EINVAL;
  if (every < 0) return fail(h, LH_EINVAL, "every < 0");
  if (every > 0 && !(maxerr >= 0.0)) return fail(h, LH_EINVAL, "maxerr must be non-negative");
  h->mon_every = every;
  h->mon_maxerr = maxerr;
  return LH_OK;
}

int lh_get_monitor(lh_handle* h, double* divmax, int32_t* err_bits) {
  if (!h) return LH_EINVAL;
  cudaSetDevice(h->device);
  if (divmax) *divmax = h->last_divmax;
  if (err_bits) {
    int e = 0;
    int rc = read_err(h, &e);
    if (rc) return rc;
    *err_bits = e;
  }
  return LH_OK;
}

// ---------------------------------------------------------------------------
// Ensembles: one CUDA graph per RK3 step for several independent handles.
// ---------------------------------------------------------------------------
struct lh_ensemble {
  std::vector<lh_handle*> hs;
  int device = 0;
  cudaStream_t origin = nullptr;
  cudaGraphExec_t graph = nullptr;
  std::vector<unsigned long long> gens;  // members' graph_gen at capture
  std::vector<cudaEvent_t> ev;  // fork event, then one join event per member
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  double last_ms = 0;
  int mode = LH_ENS_STREAMS;     // requested mode (streams: the faster at the sizes measured)
  int used = LH_ENS_STREAMS;     // mode of the captured graph
  int launches = 0;              // kernels per step in the captured graph
  std::string err;
};

namespace {
void ens_release(lh_ensemble* e) {
  if (e->graph) cudaGraphExecDestroy(e->graph);
  for (cudaEvent_t x : e->ev) cudaEventDestroy(x);
  if (e->t0) cudaEventDestroy(e->t0);
  if (e->t1) cudaEventDestroy(e->t1);
  if (e->origin) cudaStreamDestroy(e->origin);
}
int ens_fail(lh_ensemble* e, int code, const char* msg, cudaError_t ce = cudaSuccess) {
  e->err = msg;
  if (ce != cudaSuccess) { e->err += ": "; e->err += cudaGetErrorString(ce); }
  return code;
}

extern "C++" {
// Batched mode: one launch per kernel kind and slot of the substage (the bands' z-inverse, product pass and
// z-forward, assembly, canopy forcing, Thomas sweeps, flow rate, pressure solve), each covering every member
// that has that launch; the members' arguments are descriptors in one device buffer.
struct Slot {
  int kind;                          // K_*
  size_t smem;
  std::vector<unsigned char> param;  // the Batch<D> kernel parameter
};

// Appends the slots of one kernel kind from the members' descriptors (members without the launch pass none):
// one launch per distinct dynamic shared-memory size (a launch reserves one size for all its blocks, so members
// of a larger grid class would lower the occupancy of the others), kMaxBatch members per launch.
template <typename D>
void add_slot(std::vector<Slot>& slots, int kind, const std::vector<D>& ds, const std::vector<int>& blocks,
              const std::vector<size_t>& smem) {
  std::vector<size_t> sizes(smem);
  std::sort(sizes.begin(), sizes.end());
  sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
  for (size_t sz : sizes) {
    std::vector<size_t> mine;
    for (size_t m = 0; m < ds.size(); ++m)
      if (smem[m] == sz) mine.push_back(m);
    for (size_t lo = 0; lo < mine.size(); lo += kMaxBatch) {
      const size_t n = std::min(mine.size() - lo, (size_t)kMaxBatch);
      Slot sl{};
      sl.kind = kind;
      sl.smem = sz;
      sl.param.assign(sizeof(Batch<D>), 0);
      Batch<D>* b = reinterpret_cast<Batch<D>*>(sl.param.data());
      b->n = (int)n;
      int tot = 0;
      for (size_t q = 0; q < n; ++q) {
        const size_t m = mine[lo + q];
        b->start[q] = tot;
        tot += blocks[m];
        b->desc[q] = ds[m];
      }
      b->start[n] = tot;
      slots.push_back(std::move(sl));
    }
  }
}

template <typename R>
void build_batched(const std::vector<lh_handle*>& hs, std::vector<Slot>& slots) {
  const size_t nm = hs.size();
  for (int k = 0; k < 3; ++k) {
    std::vector<NlBand<R>> nl(3 * nm);
    std::vector<int> nb(nm);
    for (size_t m = 0; m < nm; ++m) nb[m] = nl_bands<R>(hs[m], &nl[3 * m]);
    for (int b = 0; b < 3; ++b) {
      for (int part = 0; part < 3; ++part) {  // z-inverse, product pass, z-forward of band b
        std::vector<ZDesc<R>> zd;
        std::vector<XDesc<R>> xd;
        std::vector<int> blocks;
        std::vector<size_t> smem;
        for (size_t m = 0; m < nm; ++m) {
          if (nb[m] <= b) continue;
          const lh_handle* h = hs[m];
          const NlBand<R>& B = nl[3 * m + b];
          dim3 g;
          size_t sm;
          if (part == 1) {
            ProdArgs<R> xa = B.xp;
            xa.rows = 1;  // the batched launch runs one z row per CTA
            xprod_shape<R>(xa, *B.d, &g, &sm);
            if (g.x == 0) continue;
            XDesc<R> D{};
            D.a = xa; D.d = *B.d; D.ph = *B.ph; D.pf = *B.pf; D.rtw = B.rtw; D.gx = g.x; D.gy = g.y;
            xd.push_back(D);
          } else {
            const ZJobs<R>& J = part == 0 ? B.zi : B.zf;
            zpass_shape<R>(J, *B.d, h->tx, &g, &sm);
            if (g.x == 0) continue;
            ZDesc<R> D{};
            D.jobs = J; D.d = *B.d; D.p = *B.pz; D.scale = 1.0 / B.d->ngz; D.tx = h->tx;
            D.gx = g.x; D.gy = g.y; D.gz = g.z;
            zd.push_back(D);
          }
          blocks.push_back((int)(g.x * g.y * g.z));
          smem.push_back(sm);
        }
        if (part == 1) add_slot(slots, K_XPROD, xd, blocks, smem);
        else add_slot(slots, part == 0 ? K_ZINV : K_ZFWD, zd, blocks, smem);
      }
    }
    {
      std::vector<ADesc> ad;
      std::vector<int> blocks;
      for (lh_handle* h : hs) {
        ADesc D{};
        D.a = asm_args<R>(h, k); D.d = h->d; D.t = h->t;
        D.gx = (h->d.np + 255) / 256; D.gy = h->d.nyu;
        ad.push_back(D);
        blocks.push_back(D.gx * D.gy);
      }
      add_slot(slots, K_ASSEMBLE, ad, blocks, std::vector<size_t>(ad.size(), 0));
    }
    {
      std::vector<ZDesc<R>> zi, zf;
      std::vector<MDesc<R>> md;
      std::vector<int> bi, bm, bf;
      std::vector<size_t> si, sm_, sf;
      for (lh_handle* h : hs) {
        ZJobs<R> a, c;
        MaskArgs<R> mk;
        if (!ib_args<R>(h, k, &a, &mk, &c)) continue;
        dim3 g;
        size_t sm;
        zpass_shape<R>(a, h->d, h->tx, &g, &sm);
        ZDesc<R> Di{};
        Di.jobs = a; Di.d = h->d; Di.p = h->pz.plan; Di.scale = 1.0; Di.tx = h->tx; Di.gx = g.x; Di.gy = g.y; Di.gz = g.z;
        zi.push_back(Di); bi.push_back((int)(g.x * g.y * g.z)); si.push_back(sm);
        xmask_shape<R>(mk, h->d, &g, &sm);
        MDesc<R> Dm{};
        Dm.a = mk; Dm.d = h->d; Dm.ph = h->ph.plan; Dm.rtw = h->rtw; Dm.gx = g.x; Dm.gy = g.y;
        md.push_back(Dm); bm.push_back((int)(g.x * g.y)); sm_.push_back(sm);
        zpass_shape<R>(c, h->d, h->tx, &g, &sm);
        ZDesc<R> Df{};
        Df.jobs = c; Df.d = h->d; Df.p = h->pz.plan; Df.scale = 1.0 / h->d.ngz; Df.tx = h->tx;
        Df.gx = g.x; Df.gy = g.y; Df.gz = g.z;
        zf.push_back(Df); bf.push_back((int)(g.x * g.y * g.z)); sf.push_back(sm);
      }
      add_slot(slots, K_IB_ZINV, zi, bi, si);
      add_slot(slots, K_IB_XMASK, md, bm, sm_);
      add_slot(slots, K_IB_ZFWD, zf, bf, sf);
    }
    {
      std::vector<VDesc> vd;
      std::vector<FDesc> fd;
      std::vector<PDesc> pd;
      std::vector<int> bv, bfl, bp;
      for (lh_handle* h : hs) {
        VDesc V{};
        V.r1 = h->r1; V.r2 = h->r2; V.r3 = h->r3; V.u1 = h->u1; V.u2 = h->u2; V.u3 = h->u3;
        V.d = h->d; V.t = h->t; V.k = k; V.gx = (h->d.np + 127) / 128; V.gy = 3;
        vd.push_back(V); bv.push_back(V.gx * V.gy);
        if (h->prm.flag_ctpress == 0) {
          FDesc F{};
          F.u1 = h->u1; F.sc = h->sc; F.d = h->d; F.t = h->t; F.k = k; F.Qx1 = h->Qx1[k];
          fd.push_back(F); bfl.push_back(1);
        }
        PDesc P{};
        P.u1 = h->u1; P.u2 = h->u2; P.u3 = h->u3; P.p = h->p; P.psi = h->psi; P.d = h->d; P.t = h->t;
        psolve_scalars(h, k, &P.dtirk, &P.dtrk);
        P.gwb = h->gw[0][0]; P.gwt = h->gw[2][1]; P.sc = h->sc; P.gx = (h->d.np + 127) / 128;
        pd.push_back(P); bp.push_back(P.gx);
      }
      add_slot(slots, K_VSOLVE, vd, bv, std::vector<size_t>(vd.size(), 0));
      add_slot(slots, K_FLOWRATE, fd, bfl, std::vector<size_t>(fd.size(), 0));
      add_slot(slots, K_PSOLVE, pd, bp, std::vector<size_t>(pd.size(), 0));
    }
  }
}

template <typename R>
void launch_slot(const Slot& sl, cudaStream_t st) {
  const void* p = sl.param.data();
  switch (sl.kind) {
    case K_ZINV: case K_IB_ZINV: launch_zinv_batch<R>(*(const Batch<ZDesc<R>>*)p, sl.smem, st); break;
    case K_ZFWD: case K_IB_ZFWD: launch_zfwd_batch<R>(*(const Batch<ZDesc<R>>*)p, sl.smem, st); break;
    case K_XPROD: launch_xprod_batch<R>(*(const Batch<XDesc<R>>*)p, sl.smem, st); break;
    case K_IB_XMASK: launch_xmask_batch<R>(*(const Batch<MDesc<R>>*)p, sl.smem, st); break;
    case K_ASSEMBLE: launch_assemble_batch(*(const Batch<ADesc>*)p, sizeof(R) == 4, st); break;
    case K_VSOLVE: launch_vsolve_batch(*(const Batch<VDesc>*)p, st); break;
    case K_FLOWRATE: launch_flowrate_batch(*(const Batch<FDesc>*)p, st); break;
    default: launch_psolve_batch(*(const Batch<PDesc>*)p, st); break;
  }
}

// Capture of one RK3 step of every member in batched launches (the caller checked that all members share a
// precision).  Members with the same grid form a class; each class's batched launches go to a stream of their own
// (the class's first member's), forked from and joined to the origin, so that the classes' kernels overlap as
// the members' do in the streams mode.  The launch arguments live in the graph's kernel nodes.
template <typename R>
int capture_batched(lh_ensemble* e, cudaGraph_t* g) {
  std::vector<std::vector<lh_handle*>> classes;
  for (lh_handle* h : e->hs) {
    bool put = false;
    for (auto& c : classes) {
      const Dims& a = c[0]->d;
      const Dims& b = h->d;
      if (a.ngx == b.ngx && a.ngz == b.ngz && a.nyu == b.nyu && a.banded == b.banded && a.ngx2 == b.ngx2 &&
          a.ngz2 == b.ngz2) {
        c.push_back(h);
        put = true;
        break;
      }
    }
    if (!put) classes.push_back({h});
  }
  std::vector<std::vector<Slot>> slots(classes.size());
  for (size_t c = 0; c < classes.size(); ++c) build_batched<R>(classes[c], slots[c]);
  for (lh_handle* h : e->hs) {  // the members' own streams may still hold work on their fields
    const cudaError_t ce = cudaStreamSynchronize(h->st);
    if (ce != cudaSuccess) return ens_fail(e, LH_ECUDA, "member stream", ce);
  }
  cudaError_t ce = cudaStreamBeginCapture(e->origin, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) return ens_fail(e, LH_ECUDA, "capture", ce);
  cudaEventRecord(e->ev[0], e->origin);
  int launches = 0;
  for (size_t c = 0; c < classes.size(); ++c) {
    cudaStream_t st = classes[c][0]->st;
    cudaStreamWaitEvent(st, e->ev[0], 0);
    for (const Slot& sl : slots[c]) launch_slot<R>(sl, st);
    cudaEventRecord(e->ev[c + 1], st);
    cudaStreamWaitEvent(e->origin, e->ev[c + 1], 0);
    launches += (int)slots[c].size();
  }
  const cudaError_t le = cudaGetLastError();
  ce = cudaStreamEndCapture(e->origin, g);
  if (le != cudaSuccess) { if (*g) cudaGraphDestroy(*g); return ens_fail(e, LH_ECUDA, "batched launch", le); }
  if (ce != cudaSuccess) return ens_fail(e, LH_ECUDA, "capture", ce);
  e->launches = launches;
  return LH_OK;
}
}  // extern "C++"
}  // namespace

int lh_ensemble_create(lh_handle* const* hs, int32_t n, lh_ensemble** out) {
  if (!out) return LH_EINVAL;
  *out = nullptr;
  if (!hs || n < 1) return fail(nullptr, LH_EINVAL, "ensemble needs at least one handle");
  for (int i = 0; i < n; ++i) {
    if (!hs[i]) return fail(nullptr, LH_EINVAL, "NULL handle in the ensemble");
    if (hs[i]->device != hs[0]->device) return fail(nullptr, LH_EINVAL, "ensemble members must share one device");
    for (int j = 0; j < i; ++j)
      if (hs[j] == hs[i] || hs[j]->st == hs[i]->st) return fail(nullptr, LH_EINVAL, "ensemble members need distinct streams");
  }
  lh_ensemble* e = new lh_ensemble();
  e->hs.assign(hs, hs + n);
  e->device = hs[0]->device;
  cudaSetDevice(e->device);
  cudaError_t ce = cudaStreamCreateWithFlags(&e->origin, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e->t0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e->t1);
  for (int i = 0; i <= n && ce == cudaSuccess; ++i) {
    cudaEvent_t x;
    ce = cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
    if (ce == cudaSuccess) e->ev.push_back(x);
  }
  if (ce != cudaSuccess) {
    ens_release(e);
    delete e;
    return fail(nullptr, LH_ECUDA, "ensemble set-up: %s", cudaGetErrorString(ce));
  }
  *out = e;
  return LH_OK;
}

void lh_ensemble_free(lh_ensemble* e) {
  if (!e) return;
  cudaSetDevice(e->device);
  if (e->origin) cudaStreamSynchronize(e->origin);
  ens_release(e);
  delete e;
}

const char* lh_ensemble_last_error(const lh_ensemble* e) { return e ? e->err.c_str() : ""; }

int lh_ensemble_set_mode(lh_ensemble* e, int32_t mode) {
  if (!e) return LH_EINVAL;
  if (mode != LH_ENS_BATCHED && mode != LH_ENS_STREAMS) return ens_fail(e, LH_EINVAL, "unknown ensemble mode");
  if (mode != e->mode && e->graph) {
    cudaSetDevice(e->device);
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  e->mode = mode;
  return LH_OK;
}

int lh_ensemble_info(const lh_ensemble* e, int32_t* mode_used, int32_t* launches_per_step) {
  if (!e) return LH_EINVAL;
  if (mode_used) *mode_used = e->used;
  if (launches_per_step) *launches_per_step = e->launches;
  return LH_OK;
}

int lh_ensemble_step(lh_ensemble* e, int32_t nsteps, double* ms) {
  if (!e) return LH_EINVAL;
  if (nsteps < 0) return ens_fail(e, LH_EINVAL, "nsteps < 0");
  for (lh_handle* h : e->hs)
    if (!h->have_fields || !h->have_dt) return ens_fail(e, LH_ESTATE, "every member needs fields and dt");
  cudaSetDevice(e->device);
  // a member whose dt changed since the capture has new launch arguments: capture again
  bool stale = e->gens.size() != e->hs.size();
  for (size_t i = 0; !stale && i < e->hs.size(); ++i) stale = e->gens[i] != e->hs[i]->graph_gen;
  if (e->graph && stale) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  if (!e->graph) {
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaSuccess;
    bool same = true;
    for (lh_handle* h : e->hs) same = same && h->precision == e->hs[0]->precision;
    if (e->mode == LH_ENS_BATCHED && same) {
      const int rc = e->hs[0]->precision == LH_PREC_MIXED ? capture_batched<float>(e, &g) : capture_batched<double>(e, &g);
      if (rc) return rc;
      e->used = LH_ENS_BATCHED;
    } else {
      ce = cudaStreamBeginCapture(e->origin, cudaStreamCaptureModeThreadLocal);
      if (ce != cudaSuccess) return ens_fail(e, LH_ECUDA, "capture", ce);
      int rc = LH_OK;
      cudaEventRecord(e->ev[0], e->origin);
      for (size_t i = 0; i < e->hs.size() && rc == LH_OK; ++i) {
        lh_handle* h = e->hs[i];
        cudaStreamWaitEvent(h->st, e->ev[0], 0);
        for (int k = 0; k < 3 && rc == LH_OK; ++k) rc = substage(h, k, 5);
        cudaEventRecord(e->ev[i + 1], h->st);
        cudaStreamWaitEvent(e->origin, e->ev[i + 1], 0);
      }
      ce = cudaStreamEndCapture(e->origin, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return ens_fail(e, rc, "capture of a member failed");
      }
      if (ce != cudaSuccess) return ens_fail(e, LH_ECUDA, "capture", ce);
      e->used = LH_ENS_STREAMS;
      e->launches = 0;
      for (lh_handle* h : e->hs) e->launches += h->launches_per_step;
    }
    ce = cudaGraphInstantiate(&e->graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) { e->graph = nullptr; return ens_fail(e, LH_ECUDA, "instantiate", ce); }
    e->gens.clear();
    for (lh_handle* h : e->hs) e->gens.push_back(h->graph_gen);
  }
  cudaEventRecord(e->t0, e->origin);
  for (int n = 0; n < nsteps; ++n) {
    cudaError_t ce = cudaGraphLaunch(e->graph, e->origin);
    if (ce != cudaSuccess) return ens_fail(e, LH_ECUDA, "graph launch", ce);
  }
  cudaEventRecord(e->t1, e->origin);
  cudaError_t ce = cudaEventSynchronize(e->t1);
  if (ce != cudaSuccess) return ens_fail(e, LH_ECUDA, "ensemble step", ce);
  float t = 0.f;
  cudaEventElapsedTime(&t, e->t0, e->t1);
  e->last_ms = t;
  if (ms) *ms = t;
  for (lh_handle* h : e->hs) {
    h->t_now += nsteps * h->dt;
    h->iter += nsteps;
  }
  for (size_t i = 0; i < e->hs.size(); ++i) {
    int err = 0;
    if (read_err(e->hs[i], &err)) return ens_fail(e, LH_ECUDA, "reading a member's status failed");
    if (err & kErrNonFinite) {
      char msg[128];
      std::snprintf(msg, sizeof msg, "non-finite value in the fields of member %zu", i);
      return ens_fail(e, LH_ENUMERIC, msg);
    }
  }
  return LH_OK;
}

int lh_last_step_ms(lh_handle* h, double* ms, int32_t* launches) {
  if (!h) return LH_EINVAL;
  if (ms) *ms = h->last_ms;
  if (launches) *launches = h->launches_per_step;
  return LH_OK;
}

// Launch-shape autotuner: the z passes' tile width (columns per CTA) and the
// product pass's levels per CTA, each picked as the fastest of its candidates
// on this handle's grid and precision.  Only scratch buffers are written
// (mixed planes, product spectra), so the fields are untouched.
int lh_autotune(lh_handle* h, int32_t* tx_out, int32_t* chunk_out) {
  if (!h) return LH_EINVAL;
  if (!h->have_fields) return fail(h, LH_ESTATE, "fields must be set first");
  cudaSetDevice(h->device);
  CU(h, cudaStreamSynchronize(h->st));
  int optin = 0;
  CU(h, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
  const size_t elem = h->precision == LH_PREC_MIXED ? sizeof(float2) : sizeof(double2);
  cudaEvent_t e0, e1;
  CU(h, cudaEventCreate(&e0));
  CU(h, cudaEventCreate(&e1));
  const int tx0 = h->tx, ch0 = h->chunk;
  int best_tx = tx0, best_ch = ch0;
  float best = 1e30f;
  for (int tx : {1, 2, 4, 8, 16, 32}) {
    if ((size_t)h->d.ngz * tx * elem > (size_t)optin - 1024) continue;  // the z tile must fit in shared memory
    h->tx = tx;
    const float ms = h->precision == LH_PREC_MIXED ? time_parts<float>(h, true, false, e0, e1)
                                                   : time_parts<double>(h, true, false, e0, e1);
    if (ms < 0.f) { h->tx = tx0; cudaEventDestroy(e0); cudaEventDestroy(e1); return fail(h, LH_ECUDA, "autotune: z passes failed"); }
    if (ms < best) { best = ms; best_tx = tx; }
  }
  h->tx = best_tx;
  // threads per z-pass CTA at that width
  {
    const int zt0 = h->zthreads;
    float t2[2] = {0.f, 0.f};
    const int cand[2] = {256, 128};
    for (int c = 0; c < 2; ++c) {
      h->zthreads = cand[c];
      t2[c] = h->precision == LH_PREC_MIXED ? time_parts<float>(h, true, false, e0, e1)
                                            : time_parts<double>(h, true, false, e0, e1);
      if (t2[c] < 0.f) { h->zthreads = zt0; cudaEventDestroy(e0); cudaEventDestroy(e1); return fail(h, LH_ECUDA, "autotune: z passes failed"); }
    }
    h->zthreads = t2[1] < t2[0] ? 128 : 256;
    if (h->zthreads != zt0 && h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; ++h->graph_gen; }
  }
  best = 1e30f;
  for (int ch : {4, 8, 16, 32, 64}) {
    h->chunk = ch;
    const float ms = h->precision == LH_PREC_MIXED ? time_parts<float>(h, false, true, e0, e1)
                                                   : time_parts<double>(h, false, true, e0, e1);
    if (ms < 0.f) { h->chunk = ch0; cudaEventDestroy(e0); cudaEventDestroy(e1); return fail(h, LH_ECUDA, "autotune: product pass failed"); }
    if (ms < best) { best = ms; best_ch = ch; }
  }
  h->chunk = best_ch;
  // the x pass with the face pair transformed on its own: fewer buffer vectors, more CTAs per SM
  {
    const int xs0 = h->xsplit;
    float t2[2] = {0.f, 0.f};
    for (int xs = 0; xs < 2; ++xs) {
      h->xsplit = xs;
      t2[xs] = h->precision == LH_PREC_MIXED ? time_parts<float>(h, false, true, e0, e1)
                                             : time_parts<double>(h, false, true, e0, e1);
      if (t2[xs] < 0.f) { h->xsplit = xs0; cudaEventDestroy(e0); cudaEventDestroy(e1); return fail(h, LH_ECUDA, "autotune: product pass failed"); }
    }
    h->xsplit = t2[1] < t2[0] ? 1 : 0;
    if (h->xsplit != xs0 && h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; ++h->graph_gen; }
  }
  // threads per x-pass CTA (the transforms' stages have 100-200 butterflies, so 128 threads with twice the
  // CTAs per SM can beat 256) and, in the mixed form without the split, one or two z rows per CTA (the
  // two-row pass runs both rows' FP32 transforms in lockstep with the same arithmetic per row); both chosen
  // together, since the best block size depends on the rows per CTA
  {
    const int xt0 = h->xthreads, xr0 = h->xrows;
    const int maxrows = (h->precision == LH_PREC_MIXED && !h->xsplit) ? 2 : 1;
    float bestx = 1e30f;
    int bt = xt0, br = 1;
    for (int r = 1; r <= maxrows; ++r) {
      for (int th : {256, 128}) {
        h->xrows = r;
        h->xthreads = th;
        const float ms = h->precision == LH_PREC_MIXED ? time_parts<float>(h, false, true, e0, e1)
                                                       : time_parts<double>(h, false, true, e0, e1);
        if (ms < 0.f) {
          h->xthreads = xt0; h->xrows = xr0;
          cudaEventDestroy(e0); cudaEventDestroy(e1);
          return fail(h, LH_ECUDA, "autotune: product pass failed");
        }
        if (ms < bestx) { bestx = ms; bt = th; br = r; }
      }
    }
    h->xthreads = bt;
    h->xrows = br;
    if ((h->xthreads != xt0 || h->xrows != xr0) && h->graph) {
      cudaGraphExecDestroy(h->graph); h->graph = nullptr; ++h->graph_gen;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CU(h, cudaGetLastError());
  if (h->tx != tx0 || h->chunk != ch0) {  // the captured step carries the old launch shapes
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    ++h->graph_gen;
  }
  if (tx_out) *tx_out = h->tx;
  if (chunk_out) *chunk_out = h->chunk;
  return LH_OK;
}

int lh_get_launch_shapes(lh_handle* h, int32_t* tx, int32_t* chunk, int32_t* xsplit) {
  if (!h) return LH_EINVAL;
  if (tx) *tx = h->tx;
  if (chunk) *chunk = h->chunk;
  if (xsplit) *xsplit = h->xsplit;
  return LH_OK;
}

int lh_get_x_threads(lh_handle* h, int32_t* threads) {
  if (!h || !threads) return LH_EINVAL;
  *threads = h->xthreads;
  return LH_OK;
}

int lh_get_x_rows(lh_handle* h, int32_t* rows) {
  if (!h || !rows) return LH_EINVAL;
  *rows = (h->precision == LH_PREC_MIXED && h->xrows == 2 && !h->xsplit) ? 2 : 1;
  return LH_OK;
}

int lh_get_z_threads(lh_handle* h, int32_t* threads) {
  if (!h || !threads) return LH_EINVAL;
  *threads = h->zthreads;
  return LH_OK;
}

int lh_profile_step(lh_handle* h, double* ms_by_kind, int32_t* count_by_kind, int32_t nkinds) {
  if (!h || !ms_by_kind || !count_by_kind || nkinds < K_NKINDS) return LH_EINVAL;
  if (!h->have_fields || !h->have_dt) return fail(h, LH_ESTATE, "fields and dt must be set first");
  cudaSetDevice(h->device);
  CU(h, cudaStreamSynchronize(h->st));
  cudaEvent_t e0;
  CU(h, cudaEventCreate(&e0));
  CU(h, cudaEventRecord(e0, h->st));
  h->profiling = true;
  int rc = LH_OK;
  for (int k = 0; k < 3 && rc == LH_OK; ++k) rc = substage(h, k, 5);
  h->profiling = false;
  cudaError_t e = cudaStreamSynchronize(h->st);
  for (int i = 0; i < nkinds; ++i) { ms_by_kind[i] = 0.0; count_by_kind[i] = 0; }
  cudaEvent_t prev = e0;
  for (size_t i = 0; i < h->prof_ev.size(); ++i) {
    float ms = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, prev, h->prof_ev[i]);
    ms_by_kind[h->prof_kind[i]] += ms;
    count_by_kind[h->prof_kind[i]] += 1;
    prev = h->prof_ev[i];
  }
  for (cudaEvent_t ev : h->prof_ev) cudaEventDestroy(ev);
  h->prof_ev.clear();
  h->prof_kind.clear();
  cudaEventDestroy(e0);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(h, LH_ECUDA, "profiled step: %s", cudaGetErrorString(e));
  h->t_now += h->dt;
  h->iter += 1;
  return LH_OK;
}

int lh_divmax(lh_handle* h, double* out) {
  if (!h || !out) return LH_EINVAL;
  cudaSetDevice(h->device);
  return device_divmax(h, out);
}

int lh_cfl_dt(lh_handle* h, double cfl, double* dt_out) {
  if (!h || !dt_out) return LH_EINVAL;
  if (!h->have_fields) return fail(h, LH_ESTATE, "fields must be set first");
  cudaSetDevice(h->device);
  CU(h, cudaMemsetAsync(&h->sc->cflbits, 0, sizeof(unsigned long long), h->st));
  const Dims& d = h->d;
  auto run = [&](auto tag) {
    using R = decltype(tag);
    using T2 = cpx_t<R>;
    BandLaunch bl[3];
    const int nbl = band_launches(h, bl);
    for (int b = 0; b < nbl; ++b) {  // each centre plane at its band's resolution
      const BandLaunch& B = bl[b];
      const Dims& db = *B.d;
      const int ul = std::max(1, B.c_lo - 1), uh = B.c_hi, vl = ul, vh = std::min(d.nyv - 2, B.c_hi);
      ZJobs<R> J{};
      J.j[0] = ZJob<R>{h->u1, nullptr, (T2*)h->mixu + (size_t)ul * db.mp, nullptr, ul, uh - ul + 1};
      J.j[1] = ZJob<R>{h->u3, nullptr, (T2*)h->mixw + (size_t)ul * db.mp, nullptr, ul, uh - ul + 1};
      J.j[2] = ZJob<R>{h->u2, nullptr, (T2*)h->mixv + (size_t)vl * db.mp, nullptr, vl, vh - vl + 1};
      J.njobs = 3;
      J.maxlev = uh - ul + 1;
      launch_zinv<R>(J, db, *B.pz, h->tx, h->st);
      ProdArgs<R> a{};
      a.mu = (const T2*)h->mixu; a.mw = (const T2*)h->mixw; a.mv = (const T2*)h->mixv;
      for (int i = 0; i < 6; ++i) a.out[i] = (T2*)h->mixp[i];
      a.wc = h->t.wc; a.wf = h->t.wf; a.dyc = h->t.dyc;
      a.dxi = db.ngx / h->Lx; a.dzi = db.ngz / h->Lz;
      a.sc = h->sc; a.want_cfl = 1; a.chunk = h->chunk; a.split = h->xsplit; a.threads = h->xthreads;
      a.c_lo = B.c_lo; a.c_hi = B.c_hi; a.f_lo = B.c_lo; a.f_hi = B.c_lo - 1;  // centres only
      launch_xprod<R>(a, db, *B.ph, *B.pf, B.rtw, h->st);
    }
  };
  if (h->precision == LH_PREC_MIXED) run(0.0f);
  else run(0.0);
  DevScalars s;
  int rc = read_scalars(h, &s);
  if (rc) return rc;
  CU(h, cudaGetLastError());
  double cmax;
  unsigned long long b = s.cflbits;
  std::memcpy(&cmax, &b, sizeof cmax);
  const double dtc = cmax > 0.0 ? 1.0 / cmax : h->dtv;
  *dt_out = cfl * (dtc < h->dtv ? dtc : h->dtv);
  return LH_OK;
}

int lh_project(lh_handle* h) {
  if (!h) return LH_EINVAL;
  if (!h->have_fields) return fail(h, LH_ESTATE, "fields must be set first");
  cudaSetDevice(h->device);
  const double dt = h->have_dt ? h->dt : 1.0;
  const size_t fp = field_elems(h, 'p');
  // keep p: project with psi only
  CU(h, cudaMemcpyAsync(h->stage, h->p, fp * sizeof(double2), cudaMemcpyDeviceToDevice, h->st));
  const double dtirk = (1.0 / dt) / (h->aRK[0] + h->bRK[0]);
  const double dtrk = dt * (h->aRK[0] + h->bRK[0]);
  launch_psolve(h->u1, h->u2, h->u3, h->p, h->psi, h->d, h->t, dtirk, dtrk, h->gw[0][0], h->gw[2][1], h->sc, h->st);
  CU(h, cudaMemcpyAsync(h->p, h->stage, fp * sizeof(double2), cudaMemcpyDeviceToDevice, h->st));
  CU(h, cudaStreamSynchronize(h->st));
  CU(h, cudaGetLastError());
  if (h->prm.flag_ctpress != 1) {
    double Q;
    int rc = host_flowrate(h, &Q);
    if (rc) return rc;
    CU(h, cudaMemcpyAsync(&h->sc->QxT, &Q, sizeof Q, cudaMemcpyHostToDevice, h->st));
    CU(h, cudaStreamSynchronize(h->st));
  }
  return LH_OK;
}

int lh_spectra_accumulate(lh_handle* h) {
  if (!h) return LH_EINVAL;
  cudaSetDevice(h->device);
  launch_spectra(h->u1, h->u2, h->u3, h->p, h->spec, h->d, h->t, h->st);
  CU(h, cudaGetLastError());
  h->nspec += 1;
  return LH_OK;
}

int lh_spectra_flush(lh_handle* h, double* spU, double* spV, double* spW, double* spUV, double* spP, int32_t* count,
                     int32_t reset) {
  if (!h) return LH_EINVAL;
  cudaSetDevice(h->device);
  const size_t np = h->d.np;
  double* b = h->spec;
  const size_t nu = h->d.nyu * np, nv = h->d.nyv * np, npp = h->d.nyp * np;
  double* outs[5] = {spU, spV, spW, spUV, spP};
  const size_t lens[5] = {nu, nv, nu, nu, npp};
  size_t off = 0;
  for (int i = 0; i < 5; ++i) {
    if (outs[i]) CU(h, cudaMemcpyAsync(outs[i], b + off, lens[i] * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    off += lens[i];
  }
  if (count) *count = h->nspec;
  if (reset) {
    CU(h, cudaMemsetAsync(b, 0, off * sizeof(double), h->st));
    h->nspec = 0;
  }
  CU(h, cudaStreamSynchronize(h->st));
  return LH_OK;
}

int lh_stats_accumulate(lh_handle* h) {
  if (!h) return LH_EINVAL;
  if (!h->have_fields) return fail(h, LH_ESTATE, "fields must be set first");
  cudaSetDevice(h->device);
  // v at centres, w and omega_x at faces are staged in the right-hand-side buffers, which are dead between steps
  launch_stats(h->u1, h->u2, h->u3, h->p, h->r1, h->r3, h->r2, h->stat, h->d, h->t, h->st);
  CU(h, cudaGetLastError());
  h->nstat += 1;
  return LH_OK;
}

int lh_cond_accumulate(lh_handle* h) {
  if (!h) return LH_EINVAL;
  if (!h->have_fields) return fail(h, LH_ESTATE, "fields must be set first");
  if (!h->cond) return LH_OK;  // no canopies: nothing to accumulate
  cudaSetDevice(h->device);
  const Dims& d = h->d;
  cudaStream_t st = h->st;
  // v at centres, w and omega_x at faces staged in the right-hand-side scratch (dead between steps)
  launch_stage_itp(h->u2, h->u3, h->r1, h->r3, h->r2, d, h->t, st);
  // the FP64 mixed planes of one chunk live in the substage's mixed buffers: 2 planes (both walls) per j1; the
  // smallest of them (uv products) holds nyv planes of the handle's precision
  const size_t cb = h->precision == LH_PREC_MIXED ? sizeof(float2) : sizeof(double2);
  const int cap = (int)((size_t)d.nyv * cb / (2 * sizeof(double2)));
  if (cap < 1) return fail(h, LH_EINVAL, "no room for the conditional statistics planes");
  const size_t tile = (size_t)h->dnx * h->dnz;
  const int njmax = std::max(h->nju, std::max(h->njv, h->njp));
  double2* mx[7] = {(double2*)h->mixu, (double2*)h->mixw, (double2*)h->mixp[0], (double2*)h->mixp[1],
                    (double2*)h->mixp[2], (double2*)h->mixp[3], (double2*)h->mixp[4]};
  for (int j0 = 0; j0 < njmax; j0 += cap) {
    const int cu = std::max(0, std::min(cap, h->nju - j0)), cvv = std::max(0, std::min(cap, h->njv - j0)),
              cp = std::max(0, std::min(cap, h->njp - j0));
    ZJobs<double> J{};
    J.j[0] = ZJob<double>{h->u1, nullptr, mx[0], h->cond_ul + 2 * j0, 0, 2 * cu};
    J.j[1] = ZJob<double>{h->u3, nullptr, mx[1], h->cond_ul + 2 * j0, 0, 2 * cu};
    J.j[2] = ZJob<double>{h->r1, nullptr, mx[2], h->cond_ul + 2 * j0, 0, 2 * cu};
    J.j[3] = ZJob<double>{h->u2, nullptr, mx[3], h->cond_vl + 2 * j0, 0, 2 * cvv};
    J.j[4] = ZJob<double>{h->r3, nullptr, mx[4], h->cond_vl + 2 * j0, 0, 2 * cvv};
    J.j[5] = ZJob<double>{h->p, nullptr, mx[5], h->cond_pl + 2 * j0, 0, 2 * cp};
    J.j[6] = ZJob<double>{h->r2, nullptr, mx[6], h->cond_vl + 2 * j0, 0, 2 * cvv};
    J.njobs = 7;
    J.maxlev = 2 * std::max(cu, std::max(cvv, cp));
    launch_zinv<double>(J, d, h->pz.plan, h->tx, st);
    CondArgs a{};
    a.mix[0][0] = mx[0]; a.mix[0][1] = mx[1]; a.mix[0][2] = mx[2];
    a.mix[1][0] = mx[3]; a.mix[1][1] = mx[4]; a.mix[1][2] = mx[6];
    a.mix[2][0] = mx[5];
    a.out[0] = h->cond;
    a.out[1] = h->cond + 6 * (size_t)h->nju * tile;
    a.out[2] = a.out[1] + 3 * (size_t)h->njv * tile;
    a.outw = a.out[2] + 2 * (size_t)h->njp * tile;
    a.nj[0] = cu; a.nj[1] = cvv; a.nj[2] = cp;
    a.njtot[0] = h->nju; a.njtot[1] = h->njv; a.njtot[2] = h->njp;
    a.j0 = j0;
    a.dnx = h->dnx; a.dnz = h->dnz; a.ntx = d.ngx / h->dnx; a.ntz = d.ngz / h->dnz;
    launch_xcond(a, d, h->ph.plan, h->rtw, st);
  }
  CU(h, cudaGetLastError());
  h->ncond += 1;
  return LH_OK;
}

int lh_cond_flush(lh_handle* h, double* out, int32_t* dims, int32_t* count, int32_t reset) {
  if (!h) return LH_EINVAL;
  cudaSetDevice(h->device);
  if (dims) { dims[0] = h->nju; dims[1] = h->njv; dims[2] = h->njp; dims[3] = h->dnx; dims[4] = h->dnz; }
  if (count) *count = h->ncond;
  if (!h->cond) return LH_OK;
  const size_t n = (size_t)h->dnx * h->dnz * (6 * (size_t)h->nju + 5 * (size_t)h->njv + 2 * (size_t)h->njp);
  if (out) CU(h, cudaMemcpyAsync(out, h->cond, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  if (reset) {
    CU(h, cudaMemsetAsync(h->cond, 0, n * sizeof(double), h->st));
    h->ncond = 0;
  }
  CU(h, cudaStreamSynchronize(h->st));
  return LH_OK;
}

int lh_stats_flush(lh_handle* h, double* out, int32_t* count, int32_t reset) {
  if (!h) return LH_EINVAL;
  cudaSetDevice(h->device);
  const size_t n = 13 * (size_t)std::max(h->d.nyu, h->d.nyv);
  if (out) CU(h, cudaMemcpyAsync(out, h->stat, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  if (count) *count = h->nstat;
  if (reset) {
    CU(h, cudaMemsetAsync(h->stat, 0, n * sizeof(double), h->st));
    h->nstat = 0;
  }
  CU(h, cudaStreamSynchronize(h->st));
  return LH_OK;
}

}  // extern "C"
