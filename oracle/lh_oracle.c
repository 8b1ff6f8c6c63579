/*
 * lh_oracle.c -- CPU FP64 restatement of Littleharsh's RK3 time step.
 *
 * TEST INFRASTRUCTURE ONLY (the correctness oracle and the timed CPU
 * baseline).  See lh_oracle.h for the list of reference routines restated
 * here and for the layouts.  Every block below cites the reference lines it
 * follows; the nonlinear term is the documented reconstruction of the missing
 * FOU3D.f90 `nonlinear`.
 */
#include "lh_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_L 3.141592653589793238462643383279502884L

/* ------------------------------------------------------------------------- */
/* small helpers                                                              */
/* ------------------------------------------------------------------------- */

/* Real base, integer exponent, by binary exponentiation: the way Fortran
 * evaluates x**n for integer n. */
static double powi_(double x, int m) {
  unsigned n = (unsigned)(m < 0 ? -m : m);
  double y = (n & 1u) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n & 1u) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

static void* xcalloc(size_t n, size_t sz) {
  void* p = calloc(n ? n : 1, sz);
  if (!p) { fprintf(stderr, "lh_oracle: out of memory\n"); abort(); }
  return p;
}

/* ------------------------------------------------------------------------- */
/* input.in parser (start.f90:63-196, FORMATs at start.f90:433-436)           */
/* ------------------------------------------------------------------------- */

/* Field of `width` characters starting after `skip` characters of the record
 * (records shorter than that are blank-padded, as Fortran PAD='YES' does). */
static void field_(const char* line, int skip, int width, char* out) {
  int len = (int)strlen(line);
  while (len > 0 && (line[len - 1] == '\n' || line[len - 1] == '\r')) len--;
  for (int c = 0; c < width; ++c) {
    int pos = skip + c;
    out[c] = pos < len ? line[pos] : ' ';
  }
  out[width] = 0;
}

/* Fortran Iw input: blanks ignored, all blank -> 0. */
static int parse_int_(const char* f, int32_t* v) {
  char buf[64]; int n = 0;
  for (const char* p = f; *p; ++p) if (*p != ' ' && *p != '\t') { if (n < 63) buf[n++] = *p; }
  buf[n] = 0;
  if (n == 0) { *v = 0; return 0; }
  char* end; long x = strtol(buf, &end, 10);
  if (*end) return -1;
  *v = (int32_t)x;
  return 0;
}

/* Fortran Dw.d input (d = 1): blanks ignored; D/E/d/e or a bare sign start the
 * exponent; a mantissa without a decimal point has d implied decimals. */
static int parse_real_(const char* f, int d, double* v) {
  char buf[64]; int n = 0;
  for (const char* p = f; *p; ++p) if (*p != ' ' && *p != '\t') { if (n < 63) buf[n++] = *p; }
  buf[n] = 0;
  if (n == 0) { *v = 0.0; return 0; }
  /* split mantissa / exponent */
  int epos = -1;
  for (int i = 0; i < n; ++i) {
    char c = buf[i];
    if (c == 'd' || c == 'D' || c == 'e' || c == 'E' || c == 'q' || c == 'Q') { epos = i; break; }
    if ((c == '+' || c == '-') && i > 0) { epos = i; break; }
  }
  char mant[64], expo[64];
  int ml = epos < 0 ? n : epos;
  memcpy(mant, buf, (size_t)ml); mant[ml] = 0;
  expo[0] = 0;
  if (epos >= 0) {
    const char* e = buf + epos;
    if (isalpha((unsigned char)*e)) e++;
    strcpy(expo, e);
  }
  long ex = 0;
  if (expo[0]) { char* end; ex = strtol(expo, &end, 10); if (*end) return -1; }
  int has_dot = strchr(mant, '.') != NULL;
  char* end; double m = strtod(mant, &end);
  if (*end) return -1;
  if (!has_dot) ex -= d;
  char tmp[96];
  snprintf(tmp, sizeof tmp, "%se%ld", mant, ex);
  if (!has_dot) { *v = strtod(tmp, &end); return 0; }
  (void)m;
  *v = strtod(tmp, &end);
  return 0;
}

static void parse_str_(const char* f, char* out, int outlen) {
  /* A90 into a longer variable: left-justified, trailing blanks dropped here */
  int n = (int)strlen(f);
  while (n > 0 && f[n - 1] == ' ') n--;
  if (n >= outlen) n = outlen - 1;
  memcpy(out, f, (size_t)n);
  out[n] = 0;
}

int lho_read_input(const char* path, lho_input* in) {
  FILE* fp = fopen(path, "r");
  if (!fp) return -1;
  memset(in, 0, sizeof *in);
  char line[512], f[128];
  int rc = 0;
#define NEXT() do { if (!fgets(line, sizeof line, fp)) { rc = -2; goto done; } } while (0)
#define RD_R(var) do { NEXT(); field_(line, 7, 10, f); if (parse_real_(f, 1, &(var))) { rc = -3; goto done; } } while (0)
#define RD_I(var) do { NEXT(); field_(line, 7, 10, f); if (parse_int_(f, &(var))) { rc = -3; goto done; } } while (0)
#define RD_S(var) do { NEXT(); field_(line, 7, 90, f); parse_str_(f, var, (int)sizeof(var)); } while (0)
#define SKIP(n) do { for (int s_ = 0; s_ < (n); ++s_) NEXT(); } while (0)
  SKIP(9);
  RD_R(in->Re); SKIP(2);
  RD_R(in->alp); RD_R(in->bet);
  RD_I(in->ngalx1); RD_I(in->ngalx2); RD_I(in->ngalz1); RD_I(in->ngalz2); RD_I(in->ny);
  RD_R(in->dyq); RD_I(in->ppp); SKIP(2);
  RD_I(in->flag_init); SKIP(3);
  RD_S(in->fnameimb); SKIP(1);
  RD_S(in->dirin); RD_S(in->dirout); SKIP(2);
  RD_R(in->CFL); RD_I(in->nwrite);
  NEXT(); field_(line, 12, 5, f); if (parse_int_(f, &in->flag_ctpress)) { rc = -3; goto done; }
  SKIP(1);
  if (in->flag_ctpress == 1) { RD_R(in->mpgx); }
  else if (in->flag_ctpress == 0) { SKIP(1); }
  else { rc = -4; goto done; }                       /* 'Wrong presure flag' */
  SKIP(3);
  RD_R(in->Kib); RD_R(in->maxerr); RD_R(in->maxt); RD_R(in->maxA); in->maxA = -in->maxA;
  RD_I(in->physlim_bot); RD_I(in->physlim_top); SKIP(2);
  RD_I(in->geometry_type); SKIP(4);
  RD_I(in->ntilex); RD_I(in->ntilez);
  if (in->geometry_type != 0 && (in->ntilex <= 0 || in->ntilez <= 0)) { rc = -5; goto done; }
  RD_R(in->posth); RD_I(in->npeakx); RD_I(in->npeakz);
  RD_R(in->Lfracx); RD_R(in->Lfracz);
  RD_I(in->dsty); RD_I(in->dstx); RD_I(in->dstz);
  if (in->geometry_type == 2 && (in->npeakx <= 0 || in->npeakz <= 0)) { rc = -6; goto done; }
  if (in->geometry_type == 3 && (in->dstx <= 0 || in->dstz <= 0 || in->dsty <= 0)) { rc = -6; goto done; }
done:
  fclose(fp);
  return rc;
#undef NEXT
#undef RD_R
#undef RD_I
#undef RD_S
#undef SKIP
}

/* ------------------------------------------------------------------------- */
/* FFT: mixed radix 4/2/3, recursive decimation in time                       */
/* ------------------------------------------------------------------------- */

typedef struct fftplan {
  int n, nf, f[40];
  double* tw; /* n complex: exp(-2 pi i k / n) */
} fftplan;

static int fft_plan_init(fftplan* p, int n) {
  memset(p, 0, sizeof *p);
  p->n = n;
  int m = n;
  while (m % 4 == 0) { p->f[p->nf++] = 4; m /= 4; }
  while (m % 2 == 0) { p->f[p->nf++] = 2; m /= 2; }
  while (m % 3 == 0) { p->f[p->nf++] = 3; m /= 3; }
  if (m != 1 || n < 1) return -1;
  p->tw = (double*)xcalloc((size_t)2 * n, sizeof(double));
  for (int k = 0; k < n; ++k) {
    long double a = 2.0L * PI_L * (long double)k / (long double)n;
    p->tw[2 * k] = (double)cosl(a);
    p->tw[2 * k + 1] = -(double)sinl(a);
  }
  return 0;
}

static void fft_plan_free(fftplan* p) { free(p->tw); p->tw = NULL; }

/* out[0..n) = DFT of in[t*istride], t = 0..n-1; twiddle exponent stride N/n = tstride */
static void fft_rec_(const fftplan* pl, int n, int tstride, const double* in, int istride, double* out,
                     int sign, int fi) {
  if (n == 1) { out[0] = in[0]; out[1] = in[1]; return; }
  const int r = pl->f[fi];
  const int m = n / r;
  for (int q = 0; q < r; ++q) fft_rec_(pl, m, tstride * r, in + 2 * (size_t)q * istride, istride * r, out + 2 * (size_t)q * m, sign, fi + 1);
  const int N = pl->n;
  const double s = (double)sign;
  for (int k = 0; k < m; ++k) {
    double yr[4], yi[4];
    for (int q = 0; q < r; ++q) {
      double ar = out[2 * (q * m + k)], ai = out[2 * (q * m + k) + 1];
      if (q == 0) { yr[0] = ar; yi[0] = ai; continue; }
      int e = (int)(((long)q * k * tstride) % N);
      /* tw holds exp(-i a); the inverse uses its conjugate */
      const double wr = pl->tw[2 * e];
      const double wi = (sign < 0) ? pl->tw[2 * e + 1] : -pl->tw[2 * e + 1];
      yr[q] = ar * wr - ai * wi;
      yi[q] = ar * wi + ai * wr;
    }
    if (r == 2) {
      out[2 * k] = yr[0] + yr[1];            out[2 * k + 1] = yi[0] + yi[1];
      out[2 * (m + k)] = yr[0] - yr[1];      out[2 * (m + k) + 1] = yi[0] - yi[1];
    } else if (r == 4) {
      /* w4 = exp(sign*i*pi/2) = sign*i */
      double t0r = yr[0] + yr[2], t0i = yi[0] + yi[2];
      double t1r = yr[0] - yr[2], t1i = yi[0] - yi[2];
      double t2r = yr[1] + yr[3], t2i = yi[1] + yi[3];
      double t3r = yr[1] - yr[3], t3i = yi[1] - yi[3];
      /* sign*i * t3 */
      double ur = -s * t3i, ui = s * t3r;
      out[2 * k] = t0r + t2r;                out[2 * k + 1] = t0i + t2i;
      out[2 * (m + k)] = t1r + ur;           out[2 * (m + k) + 1] = t1i + ui;
      out[2 * (2 * m + k)] = t0r - t2r;      out[2 * (2 * m + k) + 1] = t0i - t2i;
      out[2 * (3 * m + k)] = t1r - ur;       out[2 * (3 * m + k) + 1] = t1i - ui;
    } else { /* r == 3, w3 = exp(sign*2 pi i/3) = -1/2 + sign*i*sqrt(3)/2 */
      const double c3 = -0.5, s3 = s * 0.86602540378443864676;
      double t1r = yr[1] + yr[2], t1i = yi[1] + yi[2];
      double t2r = yr[0] + c3 * t1r, t2i = yi[0] + c3 * t1i;
      double dr = yr[1] - yr[2], di = yi[1] - yi[2];
      /* i*s3*d */
      double ur = -s3 * di, ui = s3 * dr;
      out[2 * k] = yr[0] + t1r;              out[2 * k + 1] = yi[0] + t1i;
      out[2 * (m + k)] = t2r + ur;           out[2 * (m + k) + 1] = t2i + ui;
      out[2 * (2 * m + k)] = t2r - ur;       out[2 * (2 * m + k) + 1] = t2i - ui;
    }
  }
}

/* In-place complex DFT of `data` (n complex) with scratch `tmp` (n complex). */
static void fft_exec(const fftplan* pl, int sign, double* data, double* tmp) {
  fft_rec_(pl, pl->n, 1, data, 1, tmp, sign, 0);
  memcpy(data, tmp, sizeof(double) * 2 * (size_t)pl->n);
}

int lho_fft_c2c(int n, int sign, double* data) {
  fftplan pl;
  if (fft_plan_init(&pl, n)) return -1;
  double* tmp = (double*)xcalloc((size_t)2 * n, sizeof(double));
  fft_exec(&pl, sign, data, tmp);
  free(tmp);
  fft_plan_free(&pl);
  return 0;
}

/* Real transforms of even length n through a complex DFT of length n/2.
 * half: plan of length n/2; rtw: n/2+1 complex exp(-2 pi i k/n). */
typedef struct rfftplan {
  int n;
  fftplan half;
  double* rtw;
} rfftplan;

static int rfft_plan_init(rfftplan* p, int n) {
  memset(p, 0, sizeof *p);
  if (n < 2 || (n & 1)) return -1;
  p->n = n;
  if (fft_plan_init(&p->half, n / 2)) return -1;
  p->rtw = (double*)xcalloc((size_t)2 * (n / 2 + 1), sizeof(double));
  for (int k = 0; k <= n / 2; ++k) {
    long double a = 2.0L * PI_L * (long double)k / (long double)n;
    p->rtw[2 * k] = (double)cosl(a);
    p->rtw[2 * k + 1] = -(double)sinl(a);
  }
  return 0;
}

static void rfft_plan_free(rfftplan* p) { fft_plan_free(&p->half); free(p->rtw); }

/* forward: x[n] real -> X[0..n/2] complex, unnormalised, exp(-i); scratch: n+2 doubles x2 */
static void rfft_fwd(const rfftplan* p, const double* x, double* X, double* scr) {
  const int h = p->n / 2;
  double* z = scr;          /* h complex */
  double* t = scr + 2 * h;  /* h complex */
  memcpy(z, x, sizeof(double) * (size_t)p->n);
  fft_rec_(&p->half, h, 1, z, 1, t, -1, 0);
  for (int k = 0; k <= h; ++k) {
    int k1 = k % h, k2 = (h - k) % h;
    double zr = t[2 * k1], zi = t[2 * k1 + 1];
    double cr = t[2 * k2], ci = -t[2 * k2 + 1];
    double er = 0.5 * (zr + cr), ei = 0.5 * (zi + ci);
    /* O = -i (Z - conj Z2) / 2 */
    double dr = zr - cr, di = zi - ci;
    double or_ = 0.5 * di, oi = -0.5 * dr;
    double wr = p->rtw[2 * k], wi = p->rtw[2 * k + 1];
    X[2 * k] = er + (wr * or_ - wi * oi);
    X[2 * k + 1] = ei + (wr * oi + wi * or_);
  }
  X[1] = 0.0;
  X[2 * h + 1] = 0.0;
}

/* inverse: X[0..n/2] -> x[n], unnormalised, exp(+i); Im X[0], Im X[n/2] ignored */
static void rfft_inv(const rfftplan* p, const double* X, double* x, double* scr) {
  const int h = p->n / 2;
  double* Z = scr;
  double* t = scr + 2 * h;
  for (int k = 0; k < h; ++k) {
    double ar = X[2 * k], ai = (k == 0) ? 0.0 : X[2 * k + 1];
    int k2 = h - k;
    double br = X[2 * k2], bi = (k2 == h || k2 == 0) ? 0.0 : -X[2 * k2 + 1]; /* conj X[h-k] */
    double sr = ar + br, si = ai + bi;
    double dr = ar - br, di = ai - bi;
    /* i * exp(+2 pi i k/n) * d */
    double wr = p->rtw[2 * k], wi = -p->rtw[2 * k + 1];
    double qr = wr * dr - wi * di, qi = wr * di + wi * dr;
    Z[2 * k] = sr - qi;
    Z[2 * k + 1] = si + qr;
  }
  fft_rec_(&p->half, h, 1, Z, 1, t, +1, 0);
  memcpy(x, t, sizeof(double) * (size_t)p->n);
}

/* rft of rft_buff.f:24-86 for one vector: iopt<0 forward (x -> packed c, 1/n), else inverse */
int lho_rft(int n, int iopt, double* c) {
  rfftplan p;
  if (rfft_plan_init(&p, n)) return -1;
  double* scr = (double*)xcalloc((size_t)2 * n + 4, sizeof(double));
  double* X = (double*)xcalloc((size_t)n + 2, sizeof(double));
  if (iopt < 0) {
    rfft_fwd(&p, c, X, scr);
    const double dn1 = 1.0 / n;
    for (int i = 0; i < n + 2; ++i) c[i] = dn1 * X[i];
    c[1] = 0.0;
    c[n + 1] = 0.0;
  } else {
    memcpy(X, c, sizeof(double) * (size_t)(n + 2));
    rfft_inv(&p, X, c, scr);
  }
  free(scr); free(X);
  rfft_plan_free(&p);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* solver state                                                               */
/* ------------------------------------------------------------------------- */

struct lho {
  lho_config cfg;
  lho_sizes sz;
  int ngx, ngz, nx, nz, nkx, nplane;
  int ju0, ju1, jv0, jv1, jp0, jp1, nyu, nyv, nyp;
  int nn, dny;
  int flpress;
  double Re, alp, bet, ddthetavi, dtheta, dthetai, Lx, Lz;
  double gw[3][2], gwi[3][2];
  double *yu, *yv, *dthdyu, *dthdyv, *dyu2i, *dyv2i; /* offset by j0 */
  double *kx, *k2x, *kz, *k2z;
  double aRK[3], bRK[3], gRK[3], cRK[3], dRK[3];
  double dtv;
  /* canopy */
  int nibu, nibv, *ibu_j, *ibv_j;
  uint8_t *ibu_mask, *ibv_mask;
  int tipu[2], tipv[2];
  /* fields: complex interleaved, plane-major */
  double *u1, *u2, *u3, *p, *nu1, *nu2, *nu3, *r1, *r2, *r3, *ly1, *ly2, *ly3, *psi, *div;
  double *pUU, *pUW, *pWW, *pVV, *pUV, *pVW;
  double *dg1, *dg2, *dg3;  /* pressure LU per column: [j][col] */
  double t, dt, mpgx, QxT;
  int iter;
  /* transforms */
  fftplan zplan;
  rfftplan xplan;
  /* bands: resolution 1 is the middle band's (= resolution 0 without bands) */
  int banded;
  int ngx2, ngz2, nx2, nz2, nkx2;
  fftplan zplan2;
  rfftplan xplan2;
  int N30, N31, N32, N33, N40, N41, N42, N43; /* N(3,0..3), N(4,0..3) */
  uint8_t* lng;                               /* per mode of a plane: 1 = long column */
  /* statistics */
  int istat;
  double* stat;   /* 13 profiles */
  int icond, nju, njv, njp, dnx, dnz;
  double* cond;   /* conditional statistics, see lho_cond_get */
  int nspec;
  double *spU, *spV, *spW, *spUV, *spP;
  int nthreads;
};

#define CIDX(s, jj, kk, ii) (2 * (((size_t)(jj) * (s)->nz + (kk)) * (s)->nkx + (ii)))

/* Resolution of the physical plane of u level j / v level j: 0 wall bands, 1
 * middle band (planelim, start.f90:1336-1383). */
static int res_u(const lho* s, int j) { return s->banded && j > s->N41 && j <= s->N42; }
static int res_v(const lho* s, int j) { return s->banded && j > s->N31 && j <= s->N32; }

/* Where a column's y range puts level j (jlim, start.f90:1147-1175): 0 outside
 * the column, 1 interior, 2 boundary row. */
static int lev_u(const lho* s, int col, int j) {
  if (!s->banded || s->lng[col]) return (j == s->ju0 || j == s->ju1) ? 2 : 1;
  if (j == s->N40 || j == s->N41 + 1 || j == s->N42 || j == s->N43 + 1) return 2;
  return ((j > s->N40 && j <= s->N41) || (j > s->N42 && j <= s->N43)) ? 1 : 0;
}
static int lev_v(const lho* s, int col, int j) {
  if (!s->banded || s->lng[col]) return (j == s->jv0 || j == s->jv1) ? 2 : 1;
  if (j == s->N30 || j == s->N31 + 1 || j == s->N32 || j == s->N33 + 1) return 2;
  return ((j > s->N30 && j <= s->N31) || (j > s->N32 && j <= s->N33)) ? 1 : 0;
}
static int lev_p(const lho* s, int col, int j) {
  if (!s->banded || s->lng[col]) return 1;
  return ((j > s->N40 && j <= s->N41) || (j > s->N42 && j <= s->N43)) ? 1 : 0;
}

void lho_get_sizes(const lho* s, lho_sizes* out) { *out = s->sz; }

/* y_grid_canopy.f90:24-194 plus the band limits and Ny bookkeeping. */
static int build_grid(lho* s, int ny, double dyq, int ppp, double posth, double h_ny1, int N[4][5], int Ngal[4][5]) {
  const int dny = s->dny;
  int nn = ny - 1; /* nn = N(3,nband)+1 with N(3,nband) = ny-2 */
  const int j0 = -dny, jumax = nn + dny + 1, jvmax = nn + dny;
  const int nyu = jumax - j0 + 1, nyv = jvmax - j0 + 1;
  double* yu = (double*)xcalloc((size_t)nyu, sizeof(double));
  double* yv = (double*)xcalloc((size_t)nyv, sizeof(double));
  double* dthdyu = (double*)xcalloc((size_t)nyu, sizeof(double));
  double* dthdyv = (double*)xcalloc((size_t)nyv, sizeof(double));
  double* dyu2i = (double*)xcalloc((size_t)3 * nyu, sizeof(double));
  double* dyv2i = (double*)xcalloc((size_t)3 * nyv, sizeof(double));
#define YU(j) yu[(j) - j0]
#define YV(j) yv[(j) - j0]
#define DU(j) dthdyu[(j) - j0]
#define DV(j) dthdyv[(j) - j0]
#define D2U(c, j) dyu2i[3 * ((j) - j0) + (c) - 1]
#define D2V(c, j) dyv2i[3 * ((j) - j0) + (c) - 1]
  const double q = nn / 2.0;
  const double aaa = 15.0 * (dyq - 1.0) / ((8.0 * dyq + 7.0) * powi_(q, ppp));
  const double bbb = -30.0 * (dyq - 1.0) / ((8.0 * dyq + 7.0) * powi_(q, ppp - 2));
  const double ccc = 15.0 * dyq / ((8.0 * dyq + 7.0) * q);
  for (int j = 0; j <= nn - 1; ++j) {
    double a = j - q, b = j + 0.5 - q;
    YV(j) = aaa * powi_(a, ppp) / 5.0 + bbb * powi_(a, ppp - 2) / 3.0 + ccc * a;
    YU(j + 1) = aaa * powi_(b, ppp) / 5.0 + bbb * powi_(b, ppp - 2) / 3.0 + ccc * b;
    DV(j) = 1.0 / (aaa * powi_(a, ppp - 1) + bbb * powi_(a, ppp - 3) + ccc);
    DU(j + 1) = 1.0 / (aaa * powi_(b, ppp - 1) + bbb * powi_(b, ppp - 3) + ccc);
  }
  if (dny == 0) {
    double b = -0.5 - q;
    YU(0) = aaa * powi_(b, ppp) / 5.0 + bbb * powi_(b, ppp - 2) / 3.0 + ccc * b;
    DU(0) = 1.0 / (aaa * powi_(b, ppp - 1) + bbb * powi_(b, ppp - 3) + ccc);
    /* The reference leaves yv(nn) and yu(nn+1) unset when dsty=0; they are the
     * same polynomial evaluated at the top wall and its ghost. */
    double a = nn - q; b = nn + 0.5 - q;
    YV(nn) = aaa * powi_(a, ppp) / 5.0 + bbb * powi_(a, ppp - 2) / 3.0 + ccc * a;
    DV(nn) = 1.0 / (aaa * powi_(a, ppp - 1) + bbb * powi_(a, ppp - 3) + ccc);
    YU(nn + 1) = aaa * powi_(b, ppp) / 5.0 + bbb * powi_(b, ppp - 2) / 3.0 + ccc * b;
    DU(nn + 1) = 1.0 / (aaa * powi_(b, ppp - 1) + bbb * powi_(b, ppp - 3) + ccc);
  } else {
    const double grid_min = YV(1) - YV(0);
    const double aa1 = -(15.0 * (posth - grid_min * dny)) / (7.0 * pow((double)dny, 5.0));
    const double cc1 = (30.0 * (posth - grid_min * dny)) / (7.0 * pow((double)dny, 3.0));
    const double ee1 = grid_min;
    double b = -dny - 0.5;
    YU(-dny) = aa1 * powi_(b, 5) / 5.0 + cc1 * powi_(b, 3) / 3.0 + ee1 * b - 1.0;
    DU(-dny) = 1.0 / (aa1 * powi_(b, 4) + cc1 * powi_(b, 2) + ee1);
    for (int j = -dny; j <= -1; ++j) {
      double a = (double)j; b = j + 0.5;
      YV(j) = aa1 * pow(a, 5.0) / 5.0 + cc1 * pow(a, 3.0) / 3.0 + ee1 * a - 1.0;
      YU(j + 1) = aa1 * powi_(b, 5) / 5.0 + cc1 * powi_(b, 3) / 3.0 + ee1 * b - 1.0;
      DV(j) = 1.0 / (aa1 * (double)(j * j * j * j) + cc1 * (double)(j * j) + ee1);
      DU(j + 1) = 1.0 / (aa1 * powi_(b, 4) + cc1 * powi_(b, 2) + ee1);
    }
    for (int j = 0; j <= dny; ++j) {
      double a = (double)j; b = j + 0.5;
      YV(j + nn) = aa1 * pow(a, 5.0) / 5.0 + cc1 * pow(a, 3.0) / 3.0 + ee1 * a + 1.0;
      YU(j + nn + 1) = aa1 * powi_(b, 5) / 5.0 + cc1 * powi_(b, 3) / 3.0 + ee1 * b + 1.0;
      DV(j + nn) = 1.0 / (aa1 * (double)(j * j * j * j) + cc1 * (double)(j * j) + ee1);
      DU(j + nn + 1) = 1.0 / (aa1 * powi_(b, 4) + cc1 * powi_(b, 2) + ee1);
    }
  }
  /* second-derivative coefficients (y_grid_canopy.f90:114-145) */
  {
    int j = -dny;
    D2U(1, j) = 0.0; D2U(2, j) = -2.0 / powi_(YU(j + 1) - YU(j), 2); D2U(3, j) = 1.0 / powi_(YU(j + 1) - YU(j), 2);
    D2V(1, j) = 0.0; D2V(2, j) = -2.0 / powi_(YV(j + 1) - YV(j), 2); D2V(3, j) = 1.0 / powi_(YV(j + 1) - YV(j), 2);
    for (j = -dny + 1; j <= nn + dny - 1; ++j) {
      D2U(1, j) = 2.0 / ((YU(j) - YU(j - 1)) * (YU(j + 1) - YU(j - 1)));
      D2U(2, j) = -2.0 / ((YU(j + 1) - YU(j)) * (YU(j) - YU(j - 1)));
      D2U(3, j) = 2.0 / ((YU(j + 1) - YU(j)) * (YU(j + 1) - YU(j - 1)));
      D2V(1, j) = 2.0 / ((YV(j) - YV(j - 1)) * (YV(j + 1) - YV(j - 1)));
      D2V(2, j) = -2.0 / ((YV(j + 1) - YV(j)) * (YV(j) - YV(j - 1)));
      D2V(3, j) = 2.0 / ((YV(j + 1) - YV(j)) * (YV(j + 1) - YV(j - 1)));
    }
    j = nn + dny;
    D2U(1, j) = 2.0 / ((YU(j) - YU(j - 1)) * (YU(j + 1) - YU(j - 1)));
    D2U(2, j) = -2.0 / ((YU(j + 1) - YU(j)) * (YU(j) - YU(j - 1)));
    D2U(3, j) = 2.0 / ((YU(j + 1) - YU(j)) * (YU(j + 1) - YU(j - 1)));
    D2V(1, j) = 1.0 / powi_(YV(j) - YV(j - 1), 2); D2V(2, j) = -2.0 / powi_(YV(j) - YV(j - 1), 2); D2V(3, j) = 0.0;
    j = nn + dny + 1;
    D2U(1, j) = 1.0 / powi_(YU(j) - YU(j - 1), 2); D2U(2, j) = -2.0 / powi_(YU(j) - YU(j - 1), 2); D2U(3, j) = 0.0;
  }
  /* band limits (y_grid_canopy.f90:147-176) */
  nn = ny - 2;
  N[2][0] = -dny; N[3][0] = -dny;
  {
    int j = N[2][0];
    double h = YU(0) + h_ny1;
    while (j - j0 < nyu && YU(j) < h) j++;
    N[2][1] = j;
    N[2][2] = N[2][3] - j;  /* N(3,nband) still holds ny-2 here */
  }
  N[2][3] = nn + dny;
  N[3][1] = N[2][1] + 1;
  N[3][2] = N[2][2];
  N[3][3] = N[2][3] + 1;
  for (int b = 0; b <= 4; ++b) { Ngal[2][b] = N[2][b]; Ngal[3][b] = N[3][b]; }
  s->nn = nn;
  s->yu = yu; s->yv = yv; s->dthdyu = dthdyu; s->dthdyv = dthdyv; s->dyu2i = dyu2i; s->dyv2i = dyv2i;
#undef YU
#undef YV
#undef DU
#undef DV
#undef D2U
#undef D2V
  return 0;
}

#define YU(s, j) (s)->yu[(j) - (s)->ju0]
#define YV(s, j) (s)->yv[(j) - (s)->jv0]
#define DTHU(s, j) (s)->dthdyu[(j) - (s)->ju0]
#define DTHV(s, j) (s)->dthdyv[(j) - (s)->jv0]
#define D2U(s, c, j) (s)->dyu2i[3 * ((j) - (s)->ju0) + (c) - 1]
#define D2V(s, c, j) (s)->dyv2i[3 * ((j) - (s)->jv0) + (c) - 1]

/* boundary_canopies (geom_sym_canopy.f90:63-234) filtered like getbounds
 * (start.f90:780-990): points are kept on planes inside the processed ranges,
 * which exclude the walls (planelim, start.f90:1330-1378). */
static int build_canopy(lho* s, char* err, int errlen) {
  const lho_config* c = &s->cfg;
  s->nibu = s->nibv = 0;
  if (c->geometry_type != 3) return 0;
  if (c->ntilex == 0 || c->ntilez == 0) { snprintf(err, (size_t)errlen, "ntilex/ntilez equals 0"); return -1; }
  /* the reference checks both Ngal(1,1) and Ngal(2,1) against ntilez (geom_sym_canopy.f90:54,58) */
  if (s->ngx % c->ntilez != 0) { snprintf(err, (size_t)errlen, "nx not multiple of ntilex"); return -1; }
  if (s->ngz % c->ntilez != 0) { snprintf(err, (size_t)errlen, "nz not multiple of ntilez"); return -1; }
  const int dnx = s->ngx / c->ntilex, dnz = s->ngz / c->ntilez, dsty = c->dsty;
  const int Ngal43 = s->sz.Ngal[3][3], Ngal33 = s->sz.Ngal[2][3];
  const int nyu11 = -dsty + 1, nyu21 = 0, nyv11 = -dsty, nyv21 = -1;
  const int nyu12 = Ngal43 - dsty + 1, nyu22 = Ngal43;
  const int nyv12 = Ngal33 + 1 - dsty + 1, nyv22 = Ngal33 + 1;
  const int ulo = s->sz.N[3][0] + 1, uhi = s->sz.N[3][3];
  const int vlo = s->sz.N[2][0] + 1, vhi = s->sz.N[2][3];
  int pu[4] = {nyu11 > ulo ? nyu11 : ulo, nyu21 < uhi ? nyu21 : uhi, nyu12 > ulo ? nyu12 : ulo, nyu22 < uhi ? nyu22 : uhi};
  int pv[4] = {nyv11 > vlo ? nyv11 : vlo, nyv21 < vhi ? nyv21 : vhi, nyv12 > vlo ? nyv12 : vlo, nyv22 < vhi ? nyv22 : vhi};
  int nu = (pu[1] >= pu[0] ? pu[1] - pu[0] + 1 : 0) + (pu[3] >= pu[2] ? pu[3] - pu[2] + 1 : 0);
  int nv = (pv[1] >= pv[0] ? pv[1] - pv[0] + 1 : 0) + (pv[3] >= pv[2] ? pv[3] - pv[2] + 1 : 0);
  const size_t pl = (size_t)s->ngx * s->ngz;
  s->ibu_j = (int*)xcalloc((size_t)nu, sizeof(int));
  s->ibv_j = (int*)xcalloc((size_t)nv, sizeof(int));
  s->ibu_mask = (uint8_t*)xcalloc((size_t)nu * pl, 1);
  s->ibv_mask = (uint8_t*)xcalloc((size_t)nv * pl, 1);
  int n = 0;
  for (int r = 0; r < 2; ++r) for (int j = pu[2 * r]; j <= pu[2 * r + 1]; ++j) s->ibu_j[n++] = j;
  n = 0;
  for (int r = 0; r < 2; ++r) for (int j = pv[2 * r]; j <= pv[2 * r + 1]; ++j) s->ibv_j[n++] = j;
  s->nibu = nu; s->nibv = nv;
  s->tipu[0] = 0; s->tipu[1] = Ngal43 - dsty + 1;
  s->tipv[0] = -1; s->tipv[1] = Ngal33 - dsty + 2;
  /* list points: one stem (dstx x dstz x planes) replicated over ntilex x ntilez tiles */
  for (int grid = 0; grid < 2; ++grid) {
    for (int half = 0; half < 2; ++half) {
      int ja, jb, shift;
      if (grid == 0) { ja = half ? nyu12 : nyu11; jb = half ? nyu22 : nyu21; shift = 0; }
      else { ja = half ? nyv12 : nyv11; jb = half ? nyv22 : nyv21; shift = half ? -1 : 0; }
      for (int j1 = ja; j1 <= jb; ++j1) {
        int j = j1 + shift;
        int np = grid == 0 ? s->nibu : s->nibv;
        const int* pj = grid == 0 ? s->ibu_j : s->ibv_j;
        int p = -1;
        for (int q = 0; q < np; ++q) if (pj[q] == j) { p = q; break; }
        if (p < 0) continue; /* filtered out, as getbounds does */
        uint8_t* m = (grid == 0 ? s->ibu_mask : s->ibv_mask) + (size_t)p * pl;
        for (int ix = 1; ix <= c->ntilex; ++ix)
          for (int iz = 1; iz <= c->ntilez; ++iz)
            for (int i = 1; i <= c->dstx; ++i)
              for (int k = 1; k <= c->dstz; ++k) {
                int i1 = i + dnx * (ix - 1), k1 = k + dnz * (iz - 1);
                if (i1 < 1 || i1 > s->ngx || k1 < 1 || k1 > s->ngz) {
                  snprintf(err, (size_t)errlen, "canopy point outside the plane"); return -1;
                }
                m[(size_t)(k1 - 1) * s->ngx + (i1 - 1)] = 1;
              }
      }
    }
  }
  return 0;
}


/* LU_buildP + LU_decP (tridLU_3D_IB.f90:497-571,643-684) for every column. */
/* The p-level index ranges (first, last) of column col's bands: one for a
 * long column, band 1's and band 3's for a short one. */
static void p_segments(const lho* s, int col, int segs[2][2], int* ns) {
  if (!s->banded || s->lng[col]) {
    segs[0][0] = 0; segs[0][1] = s->nyp - 1; *ns = 1;
    return;
  }
  segs[0][0] = s->N40 + 1 - s->jp0; segs[0][1] = s->N41 - s->jp0;
  segs[1][0] = s->N42 + 1 - s->jp0; segs[1][1] = s->N43 - s->jp0;
  *ns = 2;
}

/* LU_buildP + LU_decP (tridLU_3D_IB.f90:497-571,643-684) per column and band. */
static void build_dg(lho* s) {
  const int np = s->nyp, nc = s->nplane;
  s->dg1 = (double*)xcalloc((size_t)np * nc, sizeof(double));
  s->dg2 = (double*)xcalloc((size_t)np * nc, sizeof(double));
  s->dg3 = (double*)xcalloc((size_t)np * nc, sizeof(double));
  const int p0 = s->jp0;
  double* Db = (double*)xcalloc((size_t)np + 2, sizeof(double)); /* index j-(p0-1) */
  double* Gb = (double*)xcalloc((size_t)np + 2, sizeof(double));
  double* Dt = (double*)xcalloc((size_t)np + 2, sizeof(double));
  double* Gt = (double*)xcalloc((size_t)np + 2, sizeof(double));
#define IX(j) ((j) - (p0 - 1))
  for (int j = p0; j <= s->jp1; ++j) {
    Db[IX(j - 1)] = -s->ddthetavi * DTHU(s, j);
    Gb[IX(j)] = -s->ddthetavi * DTHV(s, j);
    Dt[IX(j)] = s->ddthetavi * DTHU(s, j);
    Gt[IX(j + 1)] = s->ddthetavi * DTHV(s, j);
  }
  const double pin = 1.0 / powi_(YU(s, 2) - YU(s, 1), 2);
#pragma omp parallel for schedule(static)
  for (int col = 0; col < nc; ++col) {
    const int kk = col / s->nkx, i = col % s->nkx;
    const double k2x = s->k2x[i], k2z = s->k2z[kk];
    int segs[2][2], nsg;
    p_segments(s, col, segs, &nsg);
#define A1(j) s->dg1[(size_t)((j) - p0) * nc + col]
#define A2(j) s->dg2[(size_t)((j) - p0) * nc + col]
#define A3(j) s->dg3[(size_t)((j) - p0) * nc + col]
    for (int q = 0; q < nsg; ++q) {
      const int ns = segs[q][0] + p0, ne = segs[q][1] + p0;
      A2(ns) = (Dt[IX(ns)] * Gb[IX(ns)]) + k2x + k2z;
      A3(ns) = (Dt[IX(ns)] * Gt[IX(ns + 1)]);
      A2(ne) = (Db[IX(ne - 1)] * Gt[IX(ne)]) + k2x + k2z;
      A1(ne) = (Db[IX(ne - 1)] * Gb[IX(ne - 1)]);
      for (int j = ns + 1; j <= ne - 1; ++j) {
        A2(j) = (Db[IX(j - 1)] * Gt[IX(j)]) + (Dt[IX(j)] * Gb[IX(j)]) + k2x + k2z;
        A1(j) = (Db[IX(j - 1)] * Gb[IX(j - 1)]);
        A3(j) = (Dt[IX(j)] * Gt[IX(j + 1)]);
      }
      if (col == 0) { /* mode (0,0), a long column: Dirichlet row for psi (tridLU_3D_IB.f90:548-554) */
        A1(ns) = 0.0;
        A2(ns) = pin;
        A3(ns) = 0.0;
      }
      A2(ns) = 1.0 / A2(ns);
      for (int j = ns + 1; j <= ne; ++j) {
        A3(j - 1) = A3(j - 1) * A2(j - 1);
        A2(j) = 1.0 / (A2(j) - A1(j) * A3(j - 1));
      }
    }
#undef A1
#undef A2
#undef A3
  }
#undef IX
  free(Db); free(Gb); free(Dt); free(Gt);
}

void lho_destroy(lho* s) {
  if (!s) return;
  free(s->yu); free(s->yv); free(s->dthdyu); free(s->dthdyv); free(s->dyu2i); free(s->dyv2i);
  free(s->kx); free(s->k2x); free(s->kz); free(s->k2z);
  free(s->ibu_j); free(s->ibv_j); free(s->ibu_mask); free(s->ibv_mask);
  double* f[] = {s->u1, s->u2, s->u3, s->p, s->nu1, s->nu2, s->nu3, s->r1, s->r2, s->r3, s->ly1, s->ly2,
                 s->ly3, s->psi, s->div, s->pUU, s->pUW, s->pWW, s->pVV, s->pUV, s->pVW, s->dg1, s->dg2,
                 s->dg3, s->stat, s->spU, s->spV, s->spW, s->spUV, s->spP, s->cond};
  for (size_t i = 0; i < sizeof f / sizeof f[0]; ++i) free(f[i]);
  fft_plan_free(&s->zplan);
  rfft_plan_free(&s->xplan);
  fft_plan_free(&s->zplan2);
  rfft_plan_free(&s->xplan2);
  free(s->lng);
  free(s);
}

lho* lho_create(const lho_config* cfg, char* err, int errlen) {
  char dummy[8];
  if (!err) { err = dummy; errlen = (int)sizeof dummy; }
  err[0] = 0;
  lho* s = (lho*)xcalloc(1, sizeof(lho));
  s->cfg = *cfg;
  s->nthreads = cfg->nthreads;
#ifdef _OPENMP
  if (cfg->nthreads > 0) omp_set_num_threads(cfg->nthreads);
#endif
  s->Re = cfg->Re; s->alp = cfg->alp; s->bet = cfg->bet;
  s->flpress = cfg->flag_ctpress;
  s->ngx = cfg->ngalx; s->ngz = cfg->ngalz;
  if (s->ngx < 6 || s->ngz < 6 || cfg->ny < 8) { snprintf(err, (size_t)errlen, "grid too small"); lho_destroy(s); return NULL; }
  /* N = 2*(Ngal/3) (start.f90:115-118) */
  s->nx = 2 * (s->ngx / 3); s->nz = 2 * (s->ngz / 3);
  s->nkx = s->nx / 2 + 1;
  s->nplane = s->nkx * s->nz;
  if (fft_plan_init(&s->zplan, s->ngz) || rfft_plan_init(&s->xplan, s->ngx) || (s->ngx / 2) % 1) {
    snprintf(err, (size_t)errlen, "Ngal must factor into 2, 3 and 4"); lho_destroy(s); return NULL;
  }
  if ((s->ngx / 2) < s->nkx) { snprintf(err, (size_t)errlen, "bad x size"); lho_destroy(s); return NULL; }
  s->Lx = 2.0 * (double)PI_L / s->alp;
  s->Lz = 2.0 * (double)PI_L / s->bet;
  /* h_ny (start.f90:214-240) */
  double posth = cfg->posth, h_ny1;
  if (cfg->geometry_type == 0) { posth = 0.0; h_ny1 = 0.25; }
  else if (cfg->geometry_type == 3) { h_ny1 = 1.5 * posth; }
  else { snprintf(err, (size_t)errlen, "only geometry types 0 and 3 have a forcing builder"); lho_destroy(s); return NULL; }
  s->dny = cfg->dsty;
  if (s->dny < 0) { snprintf(err, (size_t)errlen, "dsty < 0"); lho_destroy(s); return NULL; }
  /* bands (start.f90:95-118): the middle band's resolution */
  s->ngx2 = cfg->ngalx2 > 0 ? cfg->ngalx2 : s->ngx;
  s->ngz2 = cfg->ngalz2 > 0 ? cfg->ngalz2 : s->ngz;
  s->banded = (s->ngx2 != s->ngx || s->ngz2 != s->ngz);
  s->nx2 = 2 * (s->ngx2 / 3); s->nz2 = 2 * (s->ngz2 / 3); s->nkx2 = s->nx2 / 2 + 1;
  if (s->ngx2 > s->ngx || s->ngz2 > s->ngz || s->ngx2 < 6 || s->ngz2 < 6) {
    snprintf(err, (size_t)errlen, "the middle band must not be finer than the wall bands"); lho_destroy(s); return NULL;
  }
  if (fft_plan_init(&s->zplan2, s->ngz2) || rfft_plan_init(&s->xplan2, s->ngx2)) {
    snprintf(err, (size_t)errlen, "Ngal must factor into 2, 3 and 4"); lho_destroy(s); return NULL;
  }
  s->lng = (uint8_t*)xcalloc((size_t)s->nplane, 1);
  for (int kk = 0; kk < s->nz; ++kk)
    for (int i = 0; i < s->nkx; ++i) {
      const int kz = kk < s->nz / 2 ? kk : kk - s->nz; /* signed kz index */
      s->lng[(size_t)kk * s->nkx + i] = (i < s->nkx2 && kz >= -s->nz2 / 2 && kz < s->nz2 / 2);
    }
  int N[4][5] = {{0}}, Ngal[4][5] = {{0}};
  Ngal[0][1] = cfg->ngalx; Ngal[0][2] = s->ngx2; Ngal[0][3] = cfg->ngalx; Ngal[0][4] = -2;
  Ngal[1][1] = cfg->ngalz; Ngal[1][2] = s->ngz2; Ngal[1][3] = cfg->ngalz; Ngal[1][4] = 0;
  Ngal[2][3] = cfg->ny - 2;
  memcpy(N, Ngal, sizeof N);
  for (int b = 1; b <= 3; ++b) { N[0][b] = 2 * (Ngal[0][b] / 3); N[1][b] = 2 * (Ngal[1][b] / 3); }
  s->dtheta = 1.0; s->dthetai = 1.0; s->ddthetavi = 1.0;
  build_grid(s, cfg->ny, cfg->dyq, cfg->ppp, posth, h_ny1, N, Ngal);
  memcpy(s->sz.N, N, sizeof N);
  memcpy(s->sz.Ngal, Ngal, sizeof Ngal);
  s->N30 = N[2][0]; s->N31 = N[2][1]; s->N32 = N[2][2]; s->N33 = N[2][3];
  s->N40 = N[3][0]; s->N41 = N[3][1]; s->N42 = N[3][2]; s->N43 = N[3][3];
  s->ju0 = N[3][0]; s->ju1 = N[3][3] + 1;
  s->jv0 = N[2][0]; s->jv1 = N[2][3] + 1;
  s->jp0 = N[3][0] + 1; s->jp1 = N[3][3];
  s->nyu = s->ju1 - s->ju0 + 1; s->nyv = s->jv1 - s->jv0 + 1; s->nyp = s->jp1 - s->jp0 + 1;
  /* def_k (start.f90:655-704) */
  s->kx = (double*)xcalloc((size_t)s->nkx, sizeof(double));
  s->k2x = (double*)xcalloc((size_t)s->nkx, sizeof(double));
  s->kz = (double*)xcalloc((size_t)s->nz, sizeof(double));
  s->k2z = (double*)xcalloc((size_t)s->nz, sizeof(double));
  for (int i = 0; i <= s->nx / 2; ++i) { s->kx[i] = s->alp * i; s->k2x[i] = -((s->alp * i) * (s->alp * i)); }
  for (int k = 1; k <= s->nz / 2; ++k) { double a = s->bet * (k - 1); s->kz[k - 1] = a; s->k2z[k - 1] = -(a * a); }
  for (int k = s->nz / 2 + 1; k <= s->nz; ++k) { double a = s->bet * (s->nz - k + 1); s->kz[k - 1] = -a; s->k2z[k - 1] = -(a * a); }
  /* RK3 coefficients (start.f90:413-427) */
  const double aR[3] = {4.0 / 15.0, 1.0 / 15.0, 1.0 / 6.0};
  const double gR[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
  const double cR[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0};
  const double dR[3] = {8.0 / 15.0, 2.0 / 15.0, 1.0 / 3.0};
  for (int k = 0; k < 3; ++k) { s->aRK[k] = aR[k]; s->bRK[k] = aR[k]; s->gRK[k] = gR[k]; s->cRK[k] = cR[k]; s->dRK[k] = dR[k]; }
  /* dtv (start.f90:431) */
  s->dtv = s->Re / (-s->k2x[s->nx / 2] - s->k2z[s->nz / 2 - 1] + 4.0 / powi_(YV(s, N[2][0] + 1) - YV(s, N[2][0]), 2));
  /* gridweighting (start.f90:497-511) */
  s->gw[0][0] = -(YV(s, N[2][0]) - YU(s, N[3][0])) / (YV(s, N[2][0]) - YU(s, N[3][0] + 1));
  s->gw[0][1] = (YU(s, N[3][1] + 1) - YV(s, N[2][1] + 1)) / (YV(s, N[2][1] + 1) - YU(s, N[3][1]));
  s->gw[1][0] = -(YV(s, N[2][0]) - YU(s, N[3][0])) / (YV(s, N[2][0]) - YU(s, N[3][0] + 1));
  s->gw[1][1] = (YU(s, N[3][3] + 1) - YV(s, N[2][3] + 1)) / (YV(s, N[2][3] + 1) - YU(s, N[3][3]));
  s->gw[2][0] = -(YV(s, N[2][2]) - YU(s, N[3][2])) / (YV(s, N[2][2]) - YU(s, N[3][2] + 1));
  s->gw[2][1] = (YU(s, N[3][3] + 1) - YV(s, N[2][3] + 1)) / (YV(s, N[2][3] + 1) - YU(s, N[3][3]));
  s->gwi[0][0] = (YU(s, N[3][0]) - YU(s, N[3][0] + 1)) / (YV(s, N[2][0]) - YU(s, N[3][0] + 1));
  s->gwi[1][0] = s->gwi[0][0];
  s->gwi[2][0] = (YU(s, N[3][2]) - YU(s, N[3][2] + 1)) / (YV(s, N[2][2]) - YU(s, N[3][2] + 1));
  s->gwi[0][1] = (YU(s, N[3][1] + 1) - YU(s, N[3][1])) / (YV(s, N[2][1] + 1) - YU(s, N[3][1]));
  s->gwi[1][1] = (YU(s, N[3][3] + 1) - YU(s, N[3][3])) / (YV(s, N[2][3] + 1) - YU(s, N[3][3]));
  s->gwi[2][1] = s->gwi[1][1];
  /* sizes */
  lho_sizes* z = &s->sz;
  z->ngx = s->ngx; z->ngz = s->ngz; z->nx = s->nx; z->nz = s->nz; z->nkx = s->nkx;
  z->ju0 = s->ju0; z->ju1 = s->ju1; z->jv0 = s->jv0; z->jv1 = s->jv1; z->jp0 = s->jp0; z->jp1 = s->jp1;
  z->nyu = s->nyu; z->nyv = s->nyv; z->nyp = s->nyp; z->nn = s->nn; z->dny = s->dny;
  if (build_canopy(s, err, errlen)) { lho_destroy(s); return NULL; }
  for (int q = 0; q < s->nibu; ++q)
    if (res_u(s, s->ibu_j[q])) { snprintf(err, (size_t)errlen, "canopy planes must lie in the wall bands"); lho_destroy(s); return NULL; }
  for (int q = 0; q < s->nibv; ++q)
    if (res_v(s, s->ibv_j[q])) { snprintf(err, (size_t)errlen, "canopy planes must lie in the wall bands"); lho_destroy(s); return NULL; }
  z->nibu_planes = s->nibu; z->nibv_planes = s->nibv;
  /* fields */
  const size_t fu = 2 * (size_t)s->nyu * s->nplane, fv = 2 * (size_t)s->nyv * s->nplane, fp = 2 * (size_t)s->nyp * s->nplane;
  s->u1 = (double*)xcalloc(fu, 8); s->u3 = (double*)xcalloc(fu, 8); s->u2 = (double*)xcalloc(fv, 8);
  s->p = (double*)xcalloc(fp, 8);
  s->nu1 = (double*)xcalloc(fu, 8); s->nu3 = (double*)xcalloc(fu, 8); s->nu2 = (double*)xcalloc(fv, 8);
  s->r1 = (double*)xcalloc(fu, 8); s->r3 = (double*)xcalloc(fu, 8); s->r2 = (double*)xcalloc(fv, 8);
  s->ly1 = (double*)xcalloc(fu, 8); s->ly3 = (double*)xcalloc(fu, 8); s->ly2 = (double*)xcalloc(fv, 8);
  s->psi = (double*)xcalloc(fp, 8); s->div = (double*)xcalloc(fp, 8);
  s->pUU = (double*)xcalloc(fu, 8); s->pUW = (double*)xcalloc(fu, 8); s->pWW = (double*)xcalloc(fu, 8);
  s->pVV = (double*)xcalloc(fu, 8); s->pUV = (double*)xcalloc(fv, 8); s->pVW = (double*)xcalloc(fv, 8);
  build_dg(s);
  s->stat = (double*)xcalloc((size_t)13 * (s->nyu > s->nyv ? s->nyu : s->nyv), sizeof(double));
  s->spU = (double*)xcalloc((size_t)s->nyu * s->nplane, 8);
  s->spV = (double*)xcalloc((size_t)s->nyv * s->nplane, 8);
  s->spW = (double*)xcalloc((size_t)s->nyu * s->nplane, 8);
  s->spUV = (double*)xcalloc((size_t)s->nyu * s->nplane, 8);
  s->spP = (double*)xcalloc((size_t)s->nyp * s->nplane, 8);
  if (cfg->geometry_type == 3) {
    s->dnx = s->ngx / cfg->ntilex;
    s->dnz = s->ngz / cfg->ntilez;
    s->nju = N[3][1] - N[3][0] + 1;
    s->njv = N[2][1] - N[2][0] + 1;
    s->njp = N[3][1] - N[3][0] - 1;
    const size_t pl = (size_t)s->dnx * s->dnz;
    s->cond = (double*)xcalloc(pl * (6 * (size_t)s->nju + 5 * (size_t)s->njv + 2 * (size_t)s->njp), 8);
  }
  return s;
}

void lho_get_grid(const lho* s, double* yu, double* yv, double* dthdyu, double* dthdyv, double* dyu2i,
                  double* dyv2i, double* gw) {
  if (yu) memcpy(yu, s->yu, sizeof(double) * s->nyu);
  if (yv) memcpy(yv, s->yv, sizeof(double) * s->nyv);
  if (dthdyu) memcpy(dthdyu, s->dthdyu, sizeof(double) * s->nyu);
  if (dthdyv) memcpy(dthdyv, s->dthdyv, sizeof(double) * s->nyv);
  if (dyu2i) memcpy(dyu2i, s->dyu2i, sizeof(double) * 3 * s->nyu);
  if (dyv2i) memcpy(dyv2i, s->dyv2i, sizeof(double) * 3 * s->nyv);
  if (gw) for (int b = 0; b < 3; ++b) for (int c = 0; c < 2; ++c) gw[c * 3 + b] = s->gw[b][c];
}

void lho_get_ib(const lho* s, int32_t* pu, uint8_t* mu, int32_t* pv, uint8_t* mv) {
  const size_t pl = (size_t)s->ngx * s->ngz;
  if (pu) for (int i = 0; i < s->nibu; ++i) pu[i] = s->ibu_j[i];
  if (mu && s->nibu) memcpy(mu, s->ibu_mask, pl * s->nibu);
  if (pv) for (int i = 0; i < s->nibv; ++i) pv[i] = s->ibv_j[i];
  if (mv && s->nibv) memcpy(mv, s->ibv_mask, pl * s->nibv);
}

void lho_set_fields(lho* s, const double* u1, const double* u2, const double* u3, const double* p) {
  const size_t fu = 2 * (size_t)s->nyu * s->nplane, fv = 2 * (size_t)s->nyv * s->nplane, fp = 2 * (size_t)s->nyp * s->nplane;
  if (u1) memcpy(s->u1, u1, fu * 8);
  if (u2) memcpy(s->u2, u2, fv * 8);
  if (u3) memcpy(s->u3, u3, fu * 8);
  if (p) memcpy(s->p, p, fp * 8);
}

void lho_get_fields(const lho* s, double* u1, double* u2, double* u3, double* p) {
  const size_t fu = 2 * (size_t)s->nyu * s->nplane, fv = 2 * (size_t)s->nyv * s->nplane, fp = 2 * (size_t)s->nyp * s->nplane;
  if (u1) memcpy(u1, s->u1, fu * 8);
  if (u2) memcpy(u2, s->u2, fv * 8);
  if (u3) memcpy(u3, s->u3, fu * 8);
  if (p) memcpy(p, s->p, fp * 8);
}

void lho_set_nonlinear(lho* s, const double* n1, const double* n2, const double* n3) {
  const size_t fu = 2 * (size_t)s->nyu * s->nplane, fv = 2 * (size_t)s->nyv * s->nplane;
  if (n1) memcpy(s->nu1, n1, fu * 8);
  if (n2) memcpy(s->nu2, n2, fv * 8);
  if (n3) memcpy(s->nu3, n3, fu * 8);
}

void lho_get_nonlinear(const lho* s, double* n1, double* n2, double* n3) {
  const size_t fu = 2 * (size_t)s->nyu * s->nplane, fv = 2 * (size_t)s->nyv * s->nplane;
  if (n1) memcpy(n1, s->nu1, fu * 8);
  if (n2) memcpy(n2, s->nu2, fv * 8);
  if (n3) memcpy(n3, s->nu3, fu * 8);
}

void lho_get_rhs(const lho* s, double* r1, double* r2, double* r3) {
  const size_t fu = 2 * (size_t)s->nyu * s->nplane, fv = 2 * (size_t)s->nyv * s->nplane;
  if (r1) memcpy(r1, s->r1, fu * 8);
  if (r2) memcpy(r2, s->r2, fv * 8);
  if (r3) memcpy(r3, s->r3, fu * 8);
}

void lho_set_scalars(lho* s, double t, double dt, double mpgx, double QxT) {
  s->t = t; s->dt = dt; s->mpgx = mpgx;
  if (QxT >= 0.0) s->QxT = QxT;
}

void lho_get_scalars(const lho* s, double* out) {
  out[0] = s->t; out[1] = s->dt; out[2] = s->mpgx; out[3] = s->QxT;
}

/* flowrateIm (littleharsh.f90:412-431): sum_{j=1}^{nn+1} (yv(j)-yv(j-1)) Re u(j) on mode (0,0) */
double lho_flowrate(const lho* s) {
  double Q = 0.0;
  for (int j = 1; j <= s->nn + 1; ++j) Q = Q + (YV(s, j) - YV(s, j - 1)) * s->u1[CIDX(s, j - s->ju0, 0, 0)];
  return Q;
}

/* ------------------------------------------------------------------------- */
/* plane transforms (the reference's four_to_phys/phys_to_four, with the 3/2  */
/* padding and the dk z-shift of start.f90:1177-1205)                         */
/* ------------------------------------------------------------------------- */

static size_t plane_scratch_len(const lho* s) {
  return 2 * (size_t)s->ngz * s->nkx + 4 * (size_t)s->ngz + (size_t)s->ngx + 2 + 2 * (size_t)s->ngx + 4;
}

/* Plane transforms at resolution r (0: wall bands, 1: middle band).  The
 * spectral plane always holds the fine mode set; resolution 1 reads and writes
 * only the long modes (kz mapped between the two FFT orders) and zeroes the
 * others on the way back. */
static void plane_to_phys_r(const lho* s, int r, const double* spec, double* phys, double* scr) {
  const int ngz = r ? s->ngz2 : s->ngz, nkx = r ? s->nkx2 : s->nkx, ngx = r ? s->ngx2 : s->ngx;
  const int nz = r ? s->nz2 : s->nz, pitch = s->nkx;
  const fftplan* zp = r ? &s->zplan2 : &s->zplan;
  const rfftplan* xp = r ? &s->xplan2 : &s->xplan;
  double* tmp = scr;
  double* col = tmp + 2 * (size_t)ngz * nkx;
  double* fsc = col + 2 * ngz;
  double* X = fsc + 2 * ngz;
  double* rsc = X + ngx + 2;
  for (int i = 0; i < nkx; ++i) {
    memset(col, 0, sizeof(double) * 2 * ngz);
    for (int kk = 0; kk < nz; ++kk) {
      const int sl = kk < nz / 2 ? kk : kk + (ngz - nz);
      const int ks = kk < nz / 2 ? kk : kk - nz + s->nz; /* row of the fine mode set */
      col[2 * sl] = spec[2 * ((size_t)ks * pitch + i)];
      col[2 * sl + 1] = spec[2 * ((size_t)ks * pitch + i) + 1];
    }
    fft_rec_(zp, ngz, 1, col, 1, fsc, +1, 0);
    for (int k = 0; k < ngz; ++k) {
      tmp[2 * ((size_t)k * nkx + i)] = fsc[2 * k];
      tmp[2 * ((size_t)k * nkx + i) + 1] = fsc[2 * k + 1];
    }
  }
  for (int k = 0; k < ngz; ++k) {
    memset(X, 0, sizeof(double) * (size_t)(ngx + 2));
    memcpy(X, tmp + 2 * (size_t)k * nkx, sizeof(double) * 2 * nkx);
    rfft_inv(xp, X, phys + (size_t)k * ngx, rsc);
  }
}

static void plane_to_spec_r(const lho* s, int r, const double* phys, double* spec, double* scr) {
  const int ngz = r ? s->ngz2 : s->ngz, nkx = r ? s->nkx2 : s->nkx, ngx = r ? s->ngx2 : s->ngx;
  const int nz = r ? s->nz2 : s->nz, pitch = s->nkx;
  const fftplan* zp = r ? &s->zplan2 : &s->zplan;
  const rfftplan* xp = r ? &s->xplan2 : &s->xplan;
  double* tmp = scr;
  double* col = tmp + 2 * (size_t)ngz * nkx;
  double* fsc = col + 2 * ngz;
  double* X = fsc + 2 * ngz;
  double* rsc = X + ngx + 2;
  const double dnx = 1.0 / ngx, dnz = 1.0 / ngz;
  if (r) memset(spec, 0, sizeof(double) * 2 * (size_t)s->nz * pitch);
  for (int k = 0; k < ngz; ++k) {
    rfft_fwd(xp, phys + (size_t)k * ngx, X, rsc);
    for (int m = 0; m < nkx; ++m) {
      tmp[2 * ((size_t)k * nkx + m)] = dnx * X[2 * m];
      tmp[2 * ((size_t)k * nkx + m) + 1] = dnx * X[2 * m + 1];
    }
    tmp[2 * (size_t)k * nkx + 1] = 0.0;
  }
  for (int i = 0; i < nkx; ++i) {
    for (int k = 0; k < ngz; ++k) {
      col[2 * k] = tmp[2 * ((size_t)k * nkx + i)];
      col[2 * k + 1] = tmp[2 * ((size_t)k * nkx + i) + 1];
    }
    fft_rec_(zp, ngz, 1, col, 1, fsc, -1, 0);
    for (int kk = 0; kk < nz; ++kk) {
      const int sl = kk < nz / 2 ? kk : kk + (ngz - nz);
      const int ks = kk < nz / 2 ? kk : kk - nz + s->nz;
      spec[2 * ((size_t)ks * pitch + i)] = dnz * fsc[2 * sl];
      spec[2 * ((size_t)ks * pitch + i) + 1] = dnz * fsc[2 * sl + 1];
    }
  }
}

static void plane_to_phys_(const lho* s, const double* spec, double* phys, double* scr) {
  plane_to_phys_r(s, 0, spec, phys, scr);
}
static void plane_to_spec_(const lho* s, const double* phys, double* spec, double* scr) {
  plane_to_spec_r(s, 0, phys, spec, scr);
}

void lho_plane_to_phys(const lho* s, const double* spec, double* phys) {
  double* scr = (double*)xcalloc(plane_scratch_len(s), sizeof(double));
  plane_to_phys_(s, spec, phys, scr);
  free(scr);
}

void lho_plane_to_spec(const lho* s, const double* phys, double* spec) {
  double* scr = (double*)xcalloc(plane_scratch_len(s), sizeof(double));
  plane_to_spec_(s, phys, spec, scr);
  free(scr);
}

/* ------------------------------------------------------------------------- */
/* RK3 substage                                                               */
/* ------------------------------------------------------------------------- */

/* RHS0_u1/u2/u3 with laplacian_U/V (littleharsh.f90:247-321,614-731):
 * r = (a/Re) Lu - c Nu_old - d grad p ; ly = y part of the Laplacian. */
static void rhs0(lho* s, int k) {
  const double C1 = s->aRK[k] / s->Re, C2 = -s->cRK[k], d = s->dRK[k];
  const int nc = s->nplane, nkx = s->nkx;
#pragma omp parallel for schedule(static)
  for (int jj = 1; jj < s->nyu - 1; ++jj) {
    const int j = jj + s->ju0;
    const double a1 = D2U(s, 1, j), a2 = D2U(s, 2, j), a3 = D2U(s, 3, j);
    const int jp = j - s->jp0;
    for (int col = 0; col < nc; ++col) {
      const int kk = col / nkx, i = col % nkx;
      const double k2 = s->k2x[i] + s->k2z[kk];
      const size_t c0 = 2 * ((size_t)jj * nc + col), cm = c0 - 2 * (size_t)nc, cp = c0 + 2 * (size_t)nc;
      const size_t pc = 2 * ((size_t)jp * nc + col);
      if (lev_u(s, col, j) != 1) { /* outside a short column, or its end row */
        s->r1[c0] = s->r1[c0 + 1] = s->r3[c0] = s->r3[c0 + 1] = 0.0;
        s->ly1[c0] = s->ly1[c0 + 1] = s->ly3[c0] = s->ly3[c0 + 1] = 0.0;
        continue;
      }
      for (int f = 0; f < 2; ++f) {
        const double* u = f == 0 ? s->u1 : s->u3;
        const double* nu = f == 0 ? s->nu1 : s->nu3;
        double* r = f == 0 ? s->r1 : s->r3;
        double* ly = f == 0 ? s->ly1 : s->ly3;
        const double kk_ = f == 0 ? s->kx[i] : s->kz[kk];
        for (int c = 0; c < 2; ++c) {
          double L = a1 * u[cm + c] + (k2 + a2) * u[c0 + c] + a3 * u[cp + c];
          ly[c0 + c] = a1 * u[cm + c] + (a2) * u[c0 + c] + a3 * u[cp + c];
          /* C3 * p with C3 = -d * i*k : (d k pi, -d k pr) */
          double gp = c == 0 ? (d * kk_) * s->p[pc + 1] : -(d * kk_) * s->p[pc];
          r[c0 + c] = C1 * L + C2 * nu[c0 + c] + gp;
        }
      }
    }
  }
  /* mean pressure gradient on mode (0,0), j = N(4,0)+1 .. N(4,nband) */
  {
    const double C = -d * s->mpgx;
    for (int jj = 1; jj < s->nyu - 1; ++jj) s->r1[2 * ((size_t)jj * nc)] = s->r1[2 * ((size_t)jj * nc)] + C;
  }
#pragma omp parallel for schedule(static)
  for (int jj = 1; jj < s->nyv - 1; ++jj) {
    const int j = jj + s->jv0;
    const double a1 = D2V(s, 1, j), a2 = D2V(s, 2, j), a3 = D2V(s, 3, j);
    const double C3 = -d * s->ddthetavi * DTHV(s, j);
    const int jp = j - s->jp0; /* p(j) and p(j+1) */
    for (int col = 0; col < nc; ++col) {
      const int kk = col / nkx, i = col % nkx;
      const double k2 = s->k2x[i] + s->k2z[kk];
      const size_t c0 = 2 * ((size_t)jj * nc + col), cm = c0 - 2 * (size_t)nc, cp = c0 + 2 * (size_t)nc;
      const size_t p0 = 2 * ((size_t)jp * nc + col), p1 = p0 + 2 * (size_t)nc;
      if (lev_v(s, col, j) != 1) {
        s->r2[c0] = s->r2[c0 + 1] = s->ly2[c0] = s->ly2[c0 + 1] = 0.0;
        continue;
      }
      for (int c = 0; c < 2; ++c) {
        double L = a1 * s->u2[cm + c] + (k2 + a2) * s->u2[c0 + c] + a3 * s->u2[cp + c];
        s->ly2[c0 + c] = a1 * s->u2[cm + c] + (a2) * s->u2[c0 + c] + a3 * s->u2[cp + c];
        s->r2[c0 + c] = C1 * L + C2 * s->nu2[c0 + c] + C3 * (s->p[p1 + c] - s->p[p0 + c]);
      }
    }
  }
}

/* Reconstructed `nonlinear` (FOU3D.f90, missing).  Divergence form on the
 * staggered grid: products uu,uw,ww,vv at centres, uv,vw at faces, formed on
 * the 3/2-padded physical grid; y-interpolation of v to centres and of u,w to
 * faces is linear in the stretched coordinate.  Nu is stored for the next
 * substage and r -= gamma*Nu.  If cflmax != NULL it receives
 * max(|u|/dx + |v|/dy + |w|/dz) over the interior centres. */
static void nonlinear(lho* s, int k, double* cflmax) {
  const int nc = s->nplane, nkx = s->nkx;
  const int nres = s->banded ? 2 : 1;
  /* physical planes of every level at each resolution in use */
  double *Uc[2] = {NULL, NULL}, *Wc[2] = {NULL, NULL}, *Vf[2] = {NULL, NULL};
  size_t PLr[2];
  for (int r = 0; r < nres; ++r) {
    PLr[r] = (size_t)(r ? s->ngx2 : s->ngx) * (r ? s->ngz2 : s->ngz);
    Uc[r] = (double*)xcalloc(PLr[r] * s->nyu, 8);
    Wc[r] = (double*)xcalloc(PLr[r] * s->nyu, 8);
    Vf[r] = (double*)xcalloc(PLr[r] * s->nyv, 8);
  }
  const size_t PL = PLr[0];
  const size_t sl = plane_scratch_len(s);
#pragma omp parallel
  {
    double* scr = (double*)xcalloc(sl, 8);
    for (int r = 0; r < nres; ++r) {
#pragma omp for schedule(dynamic)
      for (int jj = 1; jj < s->nyu - 1; ++jj) {
        plane_to_phys_r(s, r, s->u1 + 2 * (size_t)jj * nc, Uc[r] + PLr[r] * jj, scr);
        plane_to_phys_r(s, r, s->u3 + 2 * (size_t)jj * nc, Wc[r] + PLr[r] * jj, scr);
      }
#pragma omp for schedule(dynamic)
      for (int jj = 1; jj < s->nyv - 1; ++jj) plane_to_phys_r(s, r, s->u2 + 2 * (size_t)jj * nc, Vf[r] + PLr[r] * jj, scr);
    }
    free(scr);
  }
  double cmax = 0.0;
#pragma omp parallel reduction(max : cmax)
  {
    double* scr = (double*)xcalloc(sl, 8);
    double* q = (double*)xcalloc(4 * PL, 8);
#pragma omp for schedule(dynamic)
    for (int jj = 1; jj < s->nyu - 1; ++jj) {
      const int j = jj + s->ju0;
      const int r = res_u(s, j);   /* each centre plane at its band's resolution */
      const size_t P = PLr[r];
      const double dxi = (r ? s->ngx2 : s->ngx) / s->Lx, dzi = (r ? s->ngz2 : s->ngz) / s->Lz;
      const int fv = j - s->jv0; /* face j lives at v index fv, face j-1 at fv-1 */
      const double wc = (YU(s, j) - YV(s, j - 1)) / (YV(s, j) - YV(s, j - 1));
      const double dyi = 1.0 / (YV(s, j) - YV(s, j - 1));
      const double* U = Uc[r] + P * jj; const double* W = Wc[r] + P * jj;
      const double* V0 = Vf[r] + P * (fv - 1); const double* V1 = Vf[r] + P * fv;
      for (size_t n = 0; n < P; ++n) {
        const double v = V0[n] + wc * (V1[n] - V0[n]);
        q[n] = U[n] * U[n];
        q[P + n] = U[n] * W[n];
        q[2 * P + n] = W[n] * W[n];
        q[3 * P + n] = v * v;
        if (cflmax) {
          double cv = fabs(U[n]) * dxi + fabs(v) * dyi + fabs(W[n]) * dzi;
          if (cv > cmax) cmax = cv;
        }
      }
      plane_to_spec_r(s, r, q, s->pUU + 2 * (size_t)jj * nc, scr);
      plane_to_spec_r(s, r, q + P, s->pUW + 2 * (size_t)jj * nc, scr);
      plane_to_spec_r(s, r, q + 2 * P, s->pWW + 2 * (size_t)jj * nc, scr);
      plane_to_spec_r(s, r, q + 3 * P, s->pVV + 2 * (size_t)jj * nc, scr);
    }
#pragma omp for schedule(dynamic)
    for (int jj = 1; jj < s->nyv - 1; ++jj) {
      const int j = jj + s->jv0;
      const int r = res_v(s, j);   /* each face plane at its band's resolution */
      const size_t P = PLr[r];
      const int cu = j - s->ju0; /* centre j and j+1 */
      const double wf = (YV(s, j) - YU(s, j)) / (YU(s, j + 1) - YU(s, j));
      const double* U0 = Uc[r] + P * cu; const double* U1 = Uc[r] + P * (cu + 1);
      const double* W0 = Wc[r] + P * cu; const double* W1 = Wc[r] + P * (cu + 1);
      const double* V = Vf[r] + P * jj;
      for (size_t n = 0; n < P; ++n) {
        const double u = U0[n] + wf * (U1[n] - U0[n]);
        const double w = W0[n] + wf * (W1[n] - W0[n]);
        q[n] = u * V[n];
        q[P + n] = w * V[n];
      }
      plane_to_spec_r(s, r, q, s->pUV + 2 * (size_t)jj * nc, scr);
      plane_to_spec_r(s, r, q + P, s->pVW + 2 * (size_t)jj * nc, scr);
    }
    free(scr); free(q);
  }
  for (int r = 0; r < nres; ++r) { free(Uc[r]); free(Wc[r]); free(Vf[r]); }
  if (cflmax) *cflmax = cmax;
  if (k < 0) return;
  /* wall faces carry v = 0: their products vanish */
  memset(s->pUV, 0, sizeof(double) * 2 * nc);
  memset(s->pVW, 0, sizeof(double) * 2 * nc);
  memset(s->pUV + 2 * (size_t)(s->nyv - 1) * nc, 0, sizeof(double) * 2 * nc);
  memset(s->pVW + 2 * (size_t)(s->nyv - 1) * nc, 0, sizeof(double) * 2 * nc);
  const double g = s->gRK[k];
#pragma omp parallel for schedule(static)
  for (int jj = 1; jj < s->nyu - 1; ++jj) {
    const int j = jj + s->ju0;
    const int fv = j - s->jv0;
    const double c = s->ddthetavi * DTHU(s, j);
    for (int col = 0; col < nc; ++col) {
      const int kk = col / nkx, i = col % nkx;
      const double kx = s->kx[i], kz = s->kz[kk];
      const size_t c0 = 2 * ((size_t)jj * nc + col);
      const size_t f1 = 2 * ((size_t)fv * nc + col), f0 = f1 - 2 * (size_t)nc;
      if (lev_u(s, col, j) != 1) {
        s->nu1[c0] = s->nu1[c0 + 1] = s->nu3[c0] = s->nu3[c0 + 1] = 0.0;
        continue;
      }
      for (int comp = 0; comp < 2; ++comp) {
        const double* A = comp == 0 ? s->pUU : s->pUW;
        const double* B = comp == 0 ? s->pUW : s->pWW;
        const double* D = comp == 0 ? s->pUV : s->pVW;
        double* nu = comp == 0 ? s->nu1 : s->nu3;
        double* r = comp == 0 ? s->r1 : s->r3;
        const double nr = (-kx * A[c0 + 1] - kz * B[c0 + 1]) + c * (D[f1] - D[f0]);
        const double ni = (kx * A[c0] + kz * B[c0]) + c * (D[f1 + 1] - D[f0 + 1]);
        nu[c0] = nr; nu[c0 + 1] = ni;
        r[c0] = r[c0] - g * nr;
        r[c0 + 1] = r[c0 + 1] - g * ni;
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int jj = 1; jj < s->nyv - 1; ++jj) {
    const int j = jj + s->jv0;
    const int cu = j - s->ju0;
    const double c = s->ddthetavi * DTHV(s, j);
    for (int col = 0; col < nc; ++col) {
      const int kk = col / nkx, i = col % nkx;
      const double kx = s->kx[i], kz = s->kz[kk];
      const size_t c0 = 2 * ((size_t)jj * nc + col);
      const size_t v0 = 2 * ((size_t)cu * nc + col), v1 = v0 + 2 * (size_t)nc;
      if (lev_v(s, col, j) != 1) {
        s->nu2[c0] = s->nu2[c0 + 1] = 0.0;
        continue;
      }
      const double nr = (-kx * s->pUV[c0 + 1] - kz * s->pVW[c0 + 1]) + c * (s->pVV[v1] - s->pVV[v0]);
      const double ni = (kx * s->pUV[c0] + kz * s->pVW[c0]) + c * (s->pVV[v1 + 1] - s->pVV[v0 + 1]);
      s->nu2[c0] = nr; s->nu2[c0 + 1] = ni;
      s->r2[c0] = s->r2[c0] - g * nr;
      s->r2[c0 + 1] = s->r2[c0 + 1] - g * ni;
    }
  }
}

/* solveU/solveV first half (littleharsh.f90:746-757,793-804) and the axz
 * division of LUsolU/LUsolV (tridLU_3D_IB.f90:90-98,165-173). */
static void implicit_rhs(lho* s, double* r, const double* u, int grid, double beta) {
  const int nc = s->nplane, nkx = s->nkx;
  const int ny = grid == 0 ? s->nyu : s->nyv, j0 = grid == 0 ? s->ju0 : s->jv0;
  const double dt = s->dt;
#pragma omp parallel for schedule(static)
  for (int jj = 0; jj < ny; ++jj) {
    for (int col = 0; col < nc; ++col) {
      const size_t c0 = 2 * ((size_t)jj * nc + col);
      const int lv = grid == 0 ? lev_u(s, col, jj + j0) : lev_v(s, col, jj + j0);
      if (lv != 1) { r[c0] = 0.0; r[c0 + 1] = 0.0; continue; }  /* boundary rows and outside short columns */
      const int kk = col / nkx, i = col % nkx;
      const double axz = 1.0 - beta * (s->k2x[i] + s->k2z[kk]);
      r[c0] = (u[c0] + dt * r[c0]) / axz;
      r[c0 + 1] = (u[c0 + 1] + dt * r[c0 + 1]) / axz;
    }
  }
}

/* immersed_boundaries_U/V (tridLU_3D_IB.f90:198-359) on the processed planes. */
static void immersed(lho* s, double* r, const double* ly, int grid, double beta) {
  const int np = grid == 0 ? s->nibu : s->nibv;
  if (!np) return;
  const int* pj = grid == 0 ? s->ibu_j : s->ibv_j;
  const uint8_t* mask = grid == 0 ? s->ibu_mask : s->ibv_mask;
  const int* tip = grid == 0 ? s->tipu : s->tipv;
  const int j0 = grid == 0 ? s->ju0 : s->jv0;
  const int nc = s->nplane;
  const size_t PL = (size_t)s->ngx * s->ngz;
  const size_t sl = plane_scratch_len(s);
#pragma omp parallel
  {
    double* scr = (double*)xcalloc(sl, 8);
    double* R = (double*)xcalloc(PL, 8);
    double* L = (double*)xcalloc(PL, 8);
#pragma omp for schedule(dynamic)
    for (int q = 0; q < np; ++q) {
      const int j = pj[q];
      const size_t off = 2 * (size_t)(j - j0) * nc;
      const int is_tip = (j == tip[0] || j == tip[1]);
      plane_to_phys_(s, r + off, R, scr);
      if (is_tip) plane_to_phys_(s, ly + off, L, scr);
      const uint8_t* m = mask + PL * q;
      for (size_t n = 0; n < PL; ++n)
        if (m[n]) R[n] = is_tip ? -beta * L[n] : 0.0;
      plane_to_spec_(s, R, r + off, scr);
    }
    free(scr); free(R); free(L);
  }
}

/* LU_build + LU_dec (tridLU_3D_IB.f90:427-493,601-640) of one band's column
 * range jl..jh (global j) into a1..a3 (indexed by level), boundary rows with
 * that band's gridweighting. */
static void helm_lu(const lho* s, int grid, int band, int jl, int jh, double beta, double* a1, double* a2, double* a3) {
  const int j0 = grid == 0 ? s->ju0 : s->jv0;
  const int l = jl - j0, h = jh - j0;
  for (int jj = l + 1; jj < h; ++jj) {
    const int j = jj + j0;
    a1[jj] = -beta * (grid == 0 ? D2U(s, 1, j) : D2V(s, 1, j));
    a2[jj] = 1.0 - beta * (grid == 0 ? D2U(s, 2, j) : D2V(s, 2, j));
    a3[jj] = -beta * (grid == 0 ? D2U(s, 3, j) : D2V(s, 3, j));
  }
  a1[l] = 0.0; a2[l] = 1.0; a3[l] = grid == 0 ? s->gw[band][0] : 0.0;
  a1[h] = grid == 0 ? s->gw[band][1] : 0.0; a2[h] = 1.0; a3[h] = 0.0;
  a2[l] = 1.0 / a2[l];
  for (int jj = l + 1; jj <= h; ++jj) {
    a3[jj - 1] = a3[jj - 1] * a2[jj - 1];
    a2[jj] = 1.0 / (a2[jj] - a1[jj] * a3[jj - 1]);
  }
}

/* The Thomas sweeps of LUsolU/LUsolV (tridLU_3D_IB.f90:106-116,179-189) per
 * column over its bands: long columns over band 2's range, short columns over
 * band 1's and band 3's ranges (zero outside them). */
static void helmholtz(lho* s, double* x, int grid, double beta) {
  const int ny = grid == 0 ? s->nyu : s->nyv;
  const int j0 = grid == 0 ? s->ju0 : s->jv0;
  double* A = (double*)xcalloc((size_t)9 * ny, 8);  /* [band][3][ny] */
  helm_lu(s, grid, 1, j0, j0 + ny - 1, beta, A + 3 * ny, A + 4 * ny, A + 5 * ny);
  if (s->banded) {
    const int b1 = grid == 0 ? s->N41 + 1 : s->N31 + 1, b3 = grid == 0 ? s->N42 : s->N32;
    helm_lu(s, grid, 0, j0, b1, beta, A, A + ny, A + 2 * ny);
    helm_lu(s, grid, 2, b3, j0 + ny - 1, beta, A + 6 * ny, A + 7 * ny, A + 8 * ny);
  }
  const int nc = s->nplane;
#pragma omp parallel for schedule(static)
  for (int col = 0; col < nc; ++col) {
    int segs[2][3], ns = 0;  /* band, first, last level index */
    if (!s->banded || s->lng[col]) {
      segs[0][0] = 1; segs[0][1] = 0; segs[0][2] = ny - 1; ns = 1;
    } else {
      const int b1 = (grid == 0 ? s->N41 + 1 : s->N31 + 1) - j0, b3 = (grid == 0 ? s->N42 : s->N32) - j0;
      segs[0][0] = 0; segs[0][1] = 0; segs[0][2] = b1;
      segs[1][0] = 2; segs[1][1] = b3; segs[1][2] = ny - 1; ns = 2;
      for (int jj = b1 + 1; jj < b3; ++jj) x[2 * ((size_t)jj * nc + col)] = x[2 * ((size_t)jj * nc + col) + 1] = 0.0;
    }
    for (int q = 0; q < ns; ++q) {
      const double* a1 = A + (size_t)3 * segs[q][0] * ny;
      const double* a2 = a1 + ny;
      const double* a3 = a2 + ny;
      const int l = segs[q][1], h = segs[q][2];
      for (int c = 0; c < 2; ++c) {
#define X(jj) x[2 * ((size_t)(jj) * nc + col) + c]
        X(l) = X(l) * a2[l];
        for (int jj = l + 1; jj <= h; ++jj) X(jj) = (X(jj) - a1[jj] * X(jj - 1)) * a2[jj];
        for (int jj = h - 1; jj >= l; --jj) X(jj) = X(jj) - a3[jj] * X(jj + 1);
#undef X
      }
    }
  }
  free(A);
}

void lho_tridiag_solve(int n, const double* b1, const double* b2, const double* b3, double* x) {
  double* a2 = (double*)xcalloc((size_t)n, 8);
  double* a3 = (double*)xcalloc((size_t)n, 8);
  memcpy(a2, b2, 8 * (size_t)n); memcpy(a3, b3, 8 * (size_t)n);
  a2[0] = 1.0 / a2[0];
  for (int j = 1; j < n; ++j) { a3[j - 1] = a3[j - 1] * a2[j - 1]; a2[j] = 1.0 / (a2[j] - b1[j] * a3[j - 1]); }
  x[0] = x[0] * a2[0];
  for (int j = 1; j < n; ++j) x[j] = (x[j] - b1[j] * x[j - 1]) * a2[j];
  for (int j = n - 2; j >= 0; --j) x[j] = x[j] - a3[j] * x[j + 1];
  free(a2); free(a3);
}

/* meanflow_ctU -> flowrate_corr (littleharsh.f90:453-485,523-538) with LUsol0
 * (tridLU_3D_IB.f90:398-424,573-599,686-703) on indices 0..nn+2. */
static void flowrate_corr(lho* s, int k) {
  const int nn = s->nn, n = nn + 3;
  const double beta = s->bRK[k] * s->dt / s->Re;
  double* a1 = (double*)xcalloc((size_t)n, 8);
  double* a2 = (double*)xcalloc((size_t)n, 8);
  double* a3 = (double*)xcalloc((size_t)n, 8);
  double* u11 = (double*)xcalloc((size_t)n, 8);
  a1[0] = 0.0; a2[0] = 1.0; a3[0] = s->gw[1][0];
  for (int j = 1; j <= nn + 1; ++j) {
    a1[j] = -beta * D2U(s, 1, j);
    a2[j] = 1.0 - beta * D2U(s, 2, j);
    a3[j] = -beta * D2U(s, 3, j);
  }
  a1[nn + 2] = s->gw[1][1]; a2[nn + 2] = 1.0; a3[nn + 2] = 0.0;
  a2[0] = 1.0 / a2[0];
  for (int j = 1; j < n; ++j) { a3[j - 1] = a3[j - 1] * a2[j - 1]; a2[j] = 1.0 / (a2[j] - a1[j] * a3[j - 1]); }
  const double bdt = -s->dRK[k] * s->dt;
  u11[0] = 0.0;
  for (int j = 1; j <= nn + 1; ++j) u11[j] = bdt;
  u11[nn + 2] = 0.0;
  u11[0] = u11[0] * a2[0];
  for (int j = 1; j < n; ++j) u11[j] = (u11[j] - a1[j] * u11[j - 1]) * a2[j];
  for (int j = n - 2; j >= 0; --j) u11[j] = u11[j] - a3[j] * u11[j + 1];
  /* flowrateRe receives u11(0:) as u(1:): its u(j) is u11(j-1) */
  double Qx1 = 0.0;
  for (int j = 1; j <= nn + 1; ++j) Qx1 = Qx1 + (YV(s, j) - YV(s, j - 1)) * u11[j - 1];
  const double Qx0 = lho_flowrate(s);
  const double g = (s->QxT - Qx0) / Qx1;
  s->mpgx = s->mpgx + g;
  for (int j = 0; j <= nn + 2; ++j) {
    double* u = &s->u1[CIDX(s, j - s->ju0, 0, 0)];
    u[0] = u[0] + g * u11[j];
  }
  free(a1); free(a2); free(a3); free(u11);
}

/* divergence (littleharsh.f90:210-245) into s->div */
static void divergence(lho* s) {
  const int nc = s->nplane, nkx = s->nkx;
#pragma omp parallel for schedule(static)
  for (int jj = 0; jj < s->nyp; ++jj) {
    const int j = jj + s->jp0;
    const double c = s->ddthetavi * DTHU(s, j);
    const size_t ju = (size_t)(j - s->ju0), jv = (size_t)(j - s->jv0);
    for (int col = 0; col < nc; ++col) {
      const int kk = col / nkx, i = col % nkx;
      const double kx = s->kx[i], kz = s->kz[kk];
      const size_t cu = 2 * (ju * nc + col), cv = 2 * (jv * nc + col), cvm = cv - 2 * (size_t)nc;
      const size_t cd = 2 * ((size_t)jj * nc + col);
      if (!lev_p(s, col, j)) { s->div[cd] = s->div[cd + 1] = 0.0; continue; }
      s->div[cd] = (-kx * s->u1[cu + 1] - kz * s->u3[cu + 1]) + c * (s->u2[cv] - s->u2[cvm]);
      s->div[cd + 1] = (kx * s->u1[cu] + kz * s->u3[cu]) + c * (s->u2[cv + 1] - s->u2[cvm + 1]);
    }
  }
}

/* solveP (littleharsh.f90:557-612) with LUsolP (tridLU_3D_IB.f90:362-396),
 * then v_corr (littleharsh.f90:826-937). */
static void pressure_and_correct(lho* s, int k) {
  const int nc = s->nplane, nkx = s->nkx, np = s->nyp;
  const double dti = 1.0 / s->dt;
  const double dtirk = dti / (s->aRK[k] + s->bRK[k]);
  divergence(s);
  for (size_t n = 0; n < 2 * (size_t)np * nc; ++n) s->psi[n] = dtirk * s->div[n];
  s->psi[0] = 0.0; s->psi[1] = 0.0; /* psi(0,0) at the first p point */
#pragma omp parallel for schedule(static)
  for (int col = 0; col < nc; ++col) {
    int segs[2][2], ns;
    p_segments(s, col, segs, &ns);
    for (int q = 0; q < ns; ++q) {
      const int l = segs[q][0], h = segs[q][1];
      for (int c = 0; c < 2; ++c) {
#define X(jj) s->psi[2 * ((size_t)(jj) * nc + col) + c]
#define A(a, jj) s->a[(size_t)(jj) * nc + col]
        X(l) = X(l) * A(dg2, l);
        for (int jj = l + 1; jj <= h; ++jj) X(jj) = (X(jj) - A(dg1, jj) * X(jj - 1)) * A(dg2, jj);
        for (int jj = h - 1; jj >= l; --jj) X(jj) = X(jj) - A(dg3, jj) * X(jj + 1);
#undef X
#undef A
      }
    }
  }
  for (size_t n = 0; n < 2 * (size_t)np * nc; ++n) s->p[n] = s->p[n] + s->psi[n];
  /* v_corr */
  const double dtrk = s->dt * (s->aRK[k] + s->bRK[k]);
  const double dtrk_u2 = dtrk * s->ddthetavi;
#pragma omp parallel for schedule(static)
  for (int col = 0; col < nc; ++col) {
    const int kk = col / nkx, i = col % nkx;
    const double kx = dtrk * s->kx[i], kz = dtrk * s->kz[kk];
    for (int jj = 1; jj < s->nyu - 1; ++jj) {
      const int j = jj + s->ju0;
      if (lev_u(s, col, j) != 1) continue;
      const size_t cu = 2 * ((size_t)jj * nc + col), cp = 2 * ((size_t)(j - s->jp0) * nc + col);
      /* u -= (i kx dtrk) psi */
      s->u1[cu] = s->u1[cu] - (-kx * s->psi[cp + 1]);
      s->u1[cu + 1] = s->u1[cu + 1] - (kx * s->psi[cp]);
      s->u3[cu] = s->u3[cu] - (-kz * s->psi[cp + 1]);
      s->u3[cu + 1] = s->u3[cu + 1] - (kz * s->psi[cp]);
    }
    for (int jj = 1; jj < s->nyv - 1; ++jj) {
      const int j = jj + s->jv0;
      const size_t cv = 2 * ((size_t)jj * nc + col), cp = 2 * ((size_t)(j - s->jp0) * nc + col), cp1 = cp + 2 * (size_t)nc;
      const int lv = lev_v(s, col, j);
      if (lv != 1) {  /* v = 0 on the ends of a short column's bands (v_corr, littleharsh.f90:904-905) */
        if (lv == 2) s->u2[cv] = s->u2[cv + 1] = 0.0;
        continue;
      }
      const double f = dtrk_u2 * DTHV(s, j);
      s->u2[cv] = s->u2[cv] - f * (s->psi[cp1] - s->psi[cp]);
      s->u2[cv + 1] = s->u2[cv + 1] - f * (s->psi[cp1 + 1] - s->psi[cp + 1]);
    }
    s->u2[2 * (size_t)col] = 0.0; s->u2[2 * (size_t)col + 1] = 0.0;
    const size_t top = 2 * ((size_t)(s->nyv - 1) * nc + col);
    s->u2[top] = 0.0; s->u2[top + 1] = 0.0;
    /* ghost points from the no-slip weights */
    for (int f = 0; f < 2; ++f) {
      double* u = f == 0 ? s->u1 : s->u3;
      for (int c = 0; c < 2; ++c) {
        u[2 * (size_t)col + c] = -s->gw[0][0] * u[2 * ((size_t)nc + col) + c];
        u[2 * ((size_t)(s->nyu - 1) * nc + col) + c] = -s->gw[2][1] * u[2 * ((size_t)(s->nyu - 2) * nc + col) + c];
      }
    }
  }
  divergence(s);
}

int lho_substage(lho* s, int krk, int upto) {
  if (krk < 1 || krk > 3) return -1;
  const int k = krk - 1;
  if (!(s->dt > 0.0)) return -2;
  const double beta = s->bRK[k] * s->dt / s->Re;
  rhs0(s, k);
  nonlinear(s, k, NULL);
  implicit_rhs(s, s->r1, s->u1, 0, beta);
  implicit_rhs(s, s->r2, s->u2, 1, beta);
  implicit_rhs(s, s->r3, s->u3, 0, beta);
  if (upto <= 1) return 0;
  immersed(s, s->r1, s->ly1, 0, beta);
  immersed(s, s->r2, s->ly2, 1, beta);
  immersed(s, s->r3, s->ly3, 0, beta);
  if (upto <= 2) return 0;
  helmholtz(s, s->r1, 0, beta);
  helmholtz(s, s->r2, 1, beta);
  helmholtz(s, s->r3, 0, beta);
  {
    const size_t fu = 2 * (size_t)s->nyu * s->nplane, fv = 2 * (size_t)s->nyv * s->nplane;
    memcpy(s->u1, s->r1, fu * 8); memcpy(s->u2, s->r2, fv * 8); memcpy(s->u3, s->r3, fu * 8);
  }
  if (upto <= 3) return 0;
  if (s->flpress == 0) flowrate_corr(s, k);
  if (upto <= 4) return 0;
  pressure_and_correct(s, k);
  return 0;
}

int lho_step(lho* s, int nsteps) {
  for (int n = 0; n < nsteps; ++n) {
    for (int krk = 1; krk <= 3; ++krk) {
      int rc = lho_substage(s, krk, 5);
      if (rc) return rc;
    }
    s->t += s->dt;
    s->iter += 1;
  }
  return 0;
}

double lho_divmax(lho* s) {
  divergence(s);
  double m = 0.0;
  for (size_t n = 0; n < (size_t)s->nyp * s->nplane; ++n) {
    double a = hypot(s->div[2 * n], s->div[2 * n + 1]);
    if (a > m) m = a;
  }
  return m;
}

double lho_cfl_dt(lho* s, double cfl) {
  double cmax = 0.0;
  nonlinear(s, -1, &cmax);
  double dtc = cmax > 0.0 ? 1.0 / cmax : s->dtv;
  double d = dtc < s->dtv ? dtc : s->dtv;
  return cfl * d;
}

void lho_project(lho* s) {
  const double dt = s->dt;
  if (!(s->dt > 0.0)) s->dt = 1.0;
  const size_t fp = 2 * (size_t)s->nyp * s->nplane;
  double* p = (double*)xcalloc(fp, 8);
  memcpy(p, s->p, fp * 8);
  pressure_and_correct(s, 0);
  memcpy(s->p, p, fp * 8);
  free(p);
  s->dt = dt;
}

/* ------------------------------------------------------------------------- */
/* spectra (spectra.f90:1-56) and plane statistics (stats.f90:1-108)          */
/* ------------------------------------------------------------------------- */

/* v interpolated to the centres in spectral space; zero on the ghost centres */
static void v_to_centres(const lho* s, double* out) {
  const int nc = s->nplane;
  memset(out, 0, sizeof(double) * 2 * (size_t)s->nyu * nc);
  for (int jj = 1; jj < s->nyu - 1; ++jj) {
    const int j = jj + s->ju0;
    const double wc = (YU(s, j) - YV(s, j - 1)) / (YV(s, j) - YV(s, j - 1));
    const size_t f1 = 2 * (size_t)(j - s->jv0) * nc, f0 = f1 - 2 * (size_t)nc;
    for (size_t n = 0; n < 2 * (size_t)nc; ++n)
      out[2 * (size_t)jj * nc + n] = s->u2[f0 + n] + wc * (s->u2[f1 + n] - s->u2[f0 + n]);
  }
}

/* Streamwise vorticity omega_x = dw/dy - dv/dz on every face of the v grid
 * (the wx planes of stats.f90:53-58,93,102; the routine that fills wx lives in
 * the missing FOU3D.f90).  In spectral space per column:
 * wx(face j) = ddthetavi*dthdyv(j)*(w(centre j+1) - w(centre j)) - i kz v(face j),
 * the y-difference across the face with the metric of the pressure gradient
 * (littleharsh.f90:685). */
static void omega_x(const lho* s, double* out) {
  const int nc = s->nplane, nkx = s->nkx;
  for (int jj = 0; jj < s->nyv; ++jj) {
    const int j = jj + s->jv0;
    const double c = s->ddthetavi * DTHV(s, j);
    const size_t f = 2 * (size_t)jj * nc, c0 = 2 * (size_t)(j - s->ju0) * nc, c1 = c0 + 2 * (size_t)nc;
    for (int col = 0; col < nc; ++col) {
      const double kz = s->kz[col / nkx];
      const size_t q = 2 * (size_t)col;
      out[f + q] = c * (s->u3[c1 + q] - s->u3[c0 + q]) + kz * s->u2[f + q + 1];
      out[f + q + 1] = c * (s->u3[c1 + q + 1] - s->u3[c0 + q + 1]) - kz * s->u2[f + q];
    }
  }
}

void lho_spectra_accumulate(lho* s) {
  const int nc = s->nplane;
  double* vi = (double*)xcalloc(2 * (size_t)s->nyu * nc, 8);
  v_to_centres(s, vi);
  for (size_t n = 0; n < (size_t)s->nyu * nc; ++n) {
    s->spU[n] = s->spU[n] + s->u1[2 * n] * s->u1[2 * n] + s->u1[2 * n + 1] * s->u1[2 * n + 1];
    s->spW[n] = s->spW[n] + s->u3[2 * n] * s->u3[2 * n] + s->u3[2 * n + 1] * s->u3[2 * n + 1];
    s->spUV[n] = s->spUV[n] + s->u1[2 * n] * vi[2 * n] + s->u1[2 * n + 1] * vi[2 * n + 1];
  }
  for (size_t n = 0; n < (size_t)s->nyv * nc; ++n)
    s->spV[n] = s->spV[n] + s->u2[2 * n] * s->u2[2 * n] + s->u2[2 * n + 1] * s->u2[2 * n + 1];
  for (size_t n = 0; n < (size_t)s->nyp * nc; ++n)
    s->spP[n] = s->spP[n] + s->p[2 * n] * s->p[2 * n] + s->p[2 * n + 1] * s->p[2 * n + 1];
  s->nspec++;
  free(vi);
}

void lho_spectra_get(const lho* s, double* spU, double* spV, double* spW, double* spUV, double* spP) {
  const int nc = s->nplane;
  if (spU) memcpy(spU, s->spU, 8 * (size_t)s->nyu * nc);
  if (spV) memcpy(spV, s->spV, 8 * (size_t)s->nyv * nc);
  if (spW) memcpy(spW, s->spW, 8 * (size_t)s->nyu * nc);
  if (spUV) memcpy(spUV, s->spUV, 8 * (size_t)s->nyu * nc);
  if (spP) memcpy(spP, s->spP, 8 * (size_t)s->nyp * nc);
}

/* Profiles, stored as 13 rows of length nyu (rows on the v or p grid use the
 * first nyv / nyp entries): 0 Um, 1 U2m, 2 Vm, 3 V2m, 4 Wm, 5 W2m, 6 Pm, 7 P2m,
 * 8 UVm (u grid, v interpolated to centres), 9 UWm (u grid), 10 VWm (v grid,
 * w interpolated to faces), 11 wxm, 12 wx2m (v grid, omega_x above).  The
 * reference's wx loop runs over i <= N(1), k <= N(2) of its Ngal-sized wx
 * array, bounds left from an earlier N-grid allocation (start.f90:637-638);
 * here every plane statistic, wx's included, sums the whole physical plane. */
void lho_stats_accumulate(lho* s) {
  const int nc = s->nplane, ngx = s->ngx, ngz = s->ngz;
  const size_t PL = (size_t)ngx * ngz;
  const int L = s->nyu > s->nyv ? s->nyu : s->nyv;
  double* vi = (double*)xcalloc(2 * (size_t)s->nyu * nc, 8);
  double* wi = (double*)xcalloc(2 * (size_t)s->nyv * nc, 8);
  double* ox = (double*)xcalloc(2 * (size_t)s->nyv * nc, 8);
  v_to_centres(s, vi);
  omega_x(s, ox);
  for (int jj = 1; jj < s->nyv - 1; ++jj) {
    const int j = jj + s->jv0;
    const double wf = (YV(s, j) - YU(s, j)) / (YU(s, j + 1) - YU(s, j));
    const size_t c0 = 2 * (size_t)(j - s->ju0) * nc, c1 = c0 + 2 * (size_t)nc;
    for (size_t n = 0; n < 2 * (size_t)nc; ++n)
      wi[2 * (size_t)jj * nc + n] = s->u3[c0 + n] + wf * (s->u3[c1 + n] - s->u3[c0 + n]);
  }
  const size_t sl = plane_scratch_len(s);
#pragma omp parallel
  {
    double* scr = (double*)xcalloc(sl, 8);
    double* A = (double*)xcalloc(PL, 8);
    double* B = (double*)xcalloc(PL, 8);
#pragma omp for schedule(dynamic)
    for (int jj = 0; jj < L; ++jj) {
      double acc[13] = {0};
      /* each plane summed over its band's physical points (stats.f90 loops over N(1:2,bandPL)) */
      if (jj < s->nyu) {
        const int r = res_u(s, jj + s->ju0);
        const size_t P = r ? (size_t)s->ngx2 * s->ngz2 : PL;
        plane_to_phys_r(s, r, s->u1 + 2 * (size_t)jj * nc, A, scr);
        plane_to_phys_r(s, r, vi + 2 * (size_t)jj * nc, B, scr);
        for (size_t n = 0; n < P; ++n) { acc[0] += A[n]; acc[1] += A[n] * A[n]; acc[8] += A[n] * B[n]; }
        plane_to_phys_r(s, r, s->u3 + 2 * (size_t)jj * nc, B, scr);
        for (size_t n = 0; n < P; ++n) { acc[4] += B[n]; acc[5] += B[n] * B[n]; acc[9] += A[n] * B[n]; }
      }
      if (jj < s->nyv) {
        const int r = res_v(s, jj + s->jv0);
        const size_t P = r ? (size_t)s->ngx2 * s->ngz2 : PL;
        plane_to_phys_r(s, r, s->u2 + 2 * (size_t)jj * nc, A, scr);
        plane_to_phys_r(s, r, wi + 2 * (size_t)jj * nc, B, scr);
        for (size_t n = 0; n < P; ++n) { acc[2] += A[n]; acc[3] += A[n] * A[n]; acc[10] += A[n] * B[n]; }
        plane_to_phys_r(s, r, ox + 2 * (size_t)jj * nc, A, scr);
        for (size_t n = 0; n < P; ++n) { acc[11] += A[n]; acc[12] += A[n] * A[n]; }
      }
      if (jj < s->nyp) {
        const int r = res_u(s, jj + s->jp0);
        const size_t P = r ? (size_t)s->ngx2 * s->ngz2 : PL;
        plane_to_phys_r(s, r, s->p + 2 * (size_t)jj * nc, A, scr);
        for (size_t n = 0; n < P; ++n) { acc[6] += A[n]; acc[7] += A[n] * A[n]; }
      }
      for (int r = 0; r < 13; ++r) s->stat[(size_t)r * L + jj] += acc[r];
    }
    free(scr); free(A); free(B);
  }
  s->istat++;
  free(vi); free(wi); free(ox);
}

int lho_stats_get(const lho* s, double* out) {
  const int L = s->nyu > s->nyv ? s->nyu : s->nyv;
  memcpy(out, s->stat, sizeof(double) * 13 * (size_t)L);
  return s->istat;
}

/* Conditional statistics (conddown1/2, condup1/2: stats.f90:110-253) of the
 * wall bands, summed over both walls as recvXC does (stats.f90:473-512): the
 * bottom band's planes counted from its wall (u: j = N(4,0)+j1, v: N(3,0)+j1,
 * p: N(4,0)+1+j1) plus the top band's planes counted from the top wall
 * (u: N(4,3)+1-j1, v: N(3,3)+1-j1, p: N(4,3)-j1) with v's sign flipped.
 * Each entry sums a field over the ntilex x ntilez tiles at one in-tile point.
 * Layout of lho_cond_get's output: 13 blocks [j1][kin][i] (i fastest):
 * UmC U2mC WmC W2mC UVmC UWmC (nju planes), VmC V2mC VWmC (njv), PmC P2mC (njp),
 * wxmC wx2mC (njv; omega_x with sign +1 on both walls, as condup1 is called
 * with xsign = 1 for wx at stats.f90:102). */
void lho_cond_accumulate(lho* s) {
  if (!s->cond) return;
  const int nc = s->nplane, ngx = s->ngx, ngz = s->ngz, dnx = s->dnx, dnz = s->dnz;
  const int tx = s->cfg.ntilex, tz = s->cfg.ntilez;
  const size_t PL = (size_t)ngx * ngz, pl = (size_t)dnx * dnz;
  double* vi = (double*)xcalloc(2 * (size_t)s->nyu * nc, 8);
  double* wi = (double*)xcalloc(2 * (size_t)s->nyv * nc, 8);
  double* ox = (double*)xcalloc(2 * (size_t)s->nyv * nc, 8);
  v_to_centres(s, vi);
  omega_x(s, ox);
  for (int jj = 1; jj < s->nyv - 1; ++jj) {
    const int j = jj + s->jv0;
    const double wf = (YV(s, j) - YU(s, j)) / (YU(s, j + 1) - YU(s, j));
    const size_t c0 = 2 * (size_t)(j - s->ju0) * nc, c1 = c0 + 2 * (size_t)nc;
    for (size_t n = 0; n < 2 * (size_t)nc; ++n)
      wi[2 * (size_t)jj * nc + n] = s->u3[c0 + n] + wf * (s->u3[c1 + n] - s->u3[c0 + n]);
  }
  double* blk[13];
  blk[0] = s->cond;
  for (int q = 1; q < 13; ++q) {
    const int nj = q <= 6 ? s->nju : (q <= 9 ? s->njv : (q <= 11 ? s->njp : s->njv));  /* size of block q-1 */
    blk[q] = blk[q - 1] + (size_t)nj * pl;
  }
  const size_t sl = plane_scratch_len(s);
  double* scr = (double*)xcalloc(sl, 8);
  double* A = (double*)xcalloc(PL, 8);
  double* B = (double*)xcalloc(PL, 8);
  double* C = (double*)xcalloc(PL, 8);
  for (int side = 0; side < 2; ++side) {
    const double sg = side ? -1.0 : 1.0;
    for (int j1 = 0; j1 < s->nju; ++j1) {
      const int ju = side ? s->nyu - 1 - j1 : j1;
      plane_to_phys_(s, s->u1 + 2 * (size_t)ju * nc, A, scr);
      plane_to_phys_(s, s->u3 + 2 * (size_t)ju * nc, B, scr);
      plane_to_phys_(s, vi + 2 * (size_t)ju * nc, C, scr);
      for (int k = 0; k < dnz; ++k)
        for (int i = 0; i < dnx; ++i) {
          double a[6] = {0, 0, 0, 0, 0, 0};
          for (int iz = 0; iz < tz; ++iz)
            for (int ix = 0; ix < tx; ++ix) {
              const size_t n = (size_t)(k + dnz * iz) * ngx + i + dnx * ix;
              a[0] += A[n]; a[1] += A[n] * A[n]; a[2] += B[n]; a[3] += B[n] * B[n];
              a[4] += A[n] * (sg * C[n]); a[5] += A[n] * B[n];
            }
          for (int q = 0; q < 6; ++q) blk[q][(size_t)j1 * pl + (size_t)k * dnx + i] += a[q];
        }
    }
    for (int j1 = 0; j1 < s->njv; ++j1) {
      const int jv = side ? s->nyv - 1 - j1 : j1;
      plane_to_phys_(s, s->u2 + 2 * (size_t)jv * nc, A, scr);
      plane_to_phys_(s, wi + 2 * (size_t)jv * nc, B, scr);
      plane_to_phys_(s, ox + 2 * (size_t)jv * nc, C, scr);
      for (int k = 0; k < dnz; ++k)
        for (int i = 0; i < dnx; ++i) {
          double a[5] = {0, 0, 0, 0, 0};
          for (int iz = 0; iz < tz; ++iz)
            for (int ix = 0; ix < tx; ++ix) {
              const size_t n = (size_t)(k + dnz * iz) * ngx + i + dnx * ix;
              a[0] += sg * A[n]; a[1] += A[n] * A[n]; a[2] += (sg * A[n]) * B[n];
              a[3] += C[n]; a[4] += C[n] * C[n];
            }
          for (int q = 0; q < 3; ++q) blk[6 + q][(size_t)j1 * pl + (size_t)k * dnx + i] += a[q];
          for (int q = 0; q < 2; ++q) blk[11 + q][(size_t)j1 * pl + (size_t)k * dnx + i] += a[3 + q];
        }
    }
    for (int j1 = 0; j1 < s->njp; ++j1) {
      const int jp = side ? s->nyp - 1 - j1 : j1;
      plane_to_phys_(s, s->p + 2 * (size_t)jp * nc, A, scr);
      for (int k = 0; k < dnz; ++k)
        for (int i = 0; i < dnx; ++i) {
          double a[2] = {0, 0};
          for (int iz = 0; iz < tz; ++iz)
            for (int ix = 0; ix < tx; ++ix) {
              const size_t n = (size_t)(k + dnz * iz) * ngx + i + dnx * ix;
              a[0] += A[n]; a[1] += A[n] * A[n];
            }
          for (int q = 0; q < 2; ++q) blk[9 + q][(size_t)j1 * pl + (size_t)k * dnx + i] += a[q];
        }
    }
  }
  free(scr); free(A); free(B); free(C); free(vi); free(wi); free(ox);
  s->icond++;
}

/* out: the 13 blocks described above; returns the number of accumulations.
 * dims[0..4] = nju, njv, njp, dnx, dnz (all 0 without canopies). */
int lho_cond_get(const lho* s, double* out, int32_t* dims) {
  if (dims) { dims[0] = s->nju; dims[1] = s->njv; dims[2] = s->njp; dims[3] = s->dnx; dims[4] = s->dnz; }
  if (out && s->cond) {
    const size_t pl = (size_t)s->dnx * s->dnz;
    memcpy(out, s->cond, 8 * pl * (6 * (size_t)s->nju + 5 * (size_t)s->njv + 2 * (size_t)s->njp));
  }
  return s->icond;
}
