/*
 * lh_oracle.h -- CPU FP64 restatement of Littleharsh's RK3 time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the
 * GPU path and the timed CPU baseline.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it.  The product library never
 * links or calls it.
 *
 * What it restates (reference file:line, paths within the Littleharsh tree):
 *   - input.in parsing ........................ start.f90:63-242
 *   - stretched y grid + FD coefficients ...... y_grid_canopy.f90:24-194
 *   - wavenumbers ............................. start.f90:655-704 (def_k)
 *   - RK3 coefficients ........................ start.f90:413-427
 *   - ghost-point weights ..................... start.f90:497-503
 *   - canopy forcing lists .................... geom_sym_canopy.f90:63-234,
 *                                               filtered as getbounds does
 *                                               (start.f90:780-990) for a
 *                                               decomposition that covers
 *                                               both canopies
 *   - RHS0_u1/2/3, laplacian_U/V .............. littleharsh.f90:247-321,614-731
 *   - solveU/solveV, LUsolU/LUsolV, LU_build,
 *     LU_dec, immersed_boundaries_U/V ......... littleharsh.f90:733-824,
 *                                               tridLU_3D_IB.f90:50-359,427-493,601-640
 *   - meanflow_ctU, flowrate_corr, LUsol0 ..... littleharsh.f90:412-485,523-538,
 *                                               tridLU_3D_IB.f90:398-424,573-599,686-703
 *   - solveP, divergence, LUsolP, LU_buildP ... littleharsh.f90:210-245,557-612,
 *                                               tridLU_3D_IB.f90:362-396,497-571,643-684
 *   - v_corr .................................. littleharsh.f90:826-937
 *   - FFT normalisation and packing ........... rft_buff.f:24-86, cft_buff.f:1-65
 *   - statistics / spectra accumulation ....... stats.f90:1-253, spectra.f90:1-56
 *
 * The nonlinear term (subroutine `nonlinear`, called at littleharsh.f90:171)
 * lives in FOU3D.f90, which the reference's makefile builds but the tree does
 * not contain.  It is reconstructed here from the buffers the reference
 * declares for it (declaration.f90:78-94,151-168) as the divergence form on
 * the staggered grid with 3/2-rule dealiasing; the GPU path implements the
 * same reconstruction.  Parity with the Fortran reference itself is therefore
 * unpinned for that term; the oracle is pinned by the analytic and library
 * cross-checks in tests/.
 *
 * Layouts.  A spectral field is plane-major complex(8): [j][kk][i] with
 * i = 0..N1/2 (kx = alp*i), kk = 0..N2-1 in FFT order (kz = bet*kk for
 * kk < N2/2, bet*(kk-N2) otherwise); j runs over the field's own y range.
 * A physical plane is [k][i] real with k = 0..Ngalz-1, i = 0..Ngalx-1.
 *
 * Bands.  With two resolutions every level still holds the wall bands' (fine)
 * mode set.  Modes of the middle band's set are the long columns and live on
 * every level; the other modes are the short columns, which live only in the
 * wall bands (u: N(4,0)..N(4,1)+1 and N(4,2)..N(4,3)+1, v: N(3,0)..N(3,1)+1
 * and N(3,2)..N(3,3)+1, p: N(4,0)+1..N(4,1) and N(4,2)+1..N(4,3)) and are
 * zero elsewhere; the physical planes of the middle band (u: N(4,1)+1..N(4,2),
 * v: N(3,1)+1..N(3,2)) are transformed at the middle band's resolution.
 */
#ifndef LH_ORACLE_H
#define LH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parsed input.in (start.f90:63-196).  Strings are NUL-terminated. */
typedef struct lho_input {
  double Re, alp, bet;
  int32_t ngalx1, ngalx2, ngalz1, ngalz2, ny;
  double dyq;
  int32_t ppp;
  int32_t flag_init;
  char fnameimb[96], dirin[96], dirout[96];
  double CFL;
  int32_t nwrite, flag_ctpress;
  double mpgx;
  double Kib, maxerr, maxt, maxA;
  int32_t physlim_bot, physlim_top;
  int32_t geometry_type, ntilex, ntilez;
  double posth;
  int32_t npeakx, npeakz;
  double Lfracx, Lfracz;
  int32_t dsty, dstx, dstz;
} lho_input;

/* Configuration of one solver instance. */
typedef struct lho_config {
  double Re, alp, bet;
  int32_t ngalx, ngalz;     /* physical (dealiased) points in x and z */
  int32_t ny;               /* input.in ny */
  double dyq;
  int32_t ppp;
  int32_t geometry_type;    /* 0 smooth, 3 canopies */
  double posth;
  int32_t dsty, dstx, dstz, ntilex, ntilez;
  int32_t flag_ctpress;     /* 0 constant flow rate, 1 constant pressure gradient */
  int32_t nthreads;         /* OpenMP threads, <=0: library default */
  /* Variable-resolution bands (start.f90:95-118, 1037-1145): physical points of
   * the middle band; 0 or equal to ngalx/ngalz = one resolution everywhere.
   * ngalx/ngalz are then the wall bands' (Ngal(1:2,1) = Ngal(1:2,3)). */
  int32_t ngalx2, ngalz2;
} lho_config;

/* Sizes exposed to callers (all indices are the reference's global y indices). */
typedef struct lho_sizes {
  int32_t ngx, ngz, nx, nz, nkx;
  int32_t ju0, ju1, jv0, jv1, jp0, jp1;
  int32_t nyu, nyv, nyp;
  int32_t nn;               /* nn after y_grid_canopy (= ny-2) */
  int32_t dny;
  int32_t N[4][5], Ngal[4][5]; /* N(r+1, b) = N[r][b] */
  int32_t nibu_planes, nibv_planes;
} lho_sizes;

typedef struct lho lho;

int  lho_read_input(const char* path, lho_input* out);

lho* lho_create(const lho_config* cfg, char* err, int errlen);
void lho_destroy(lho* s);
void lho_get_sizes(const lho* s, lho_sizes* out);

/* Grid (y_grid_canopy.f90): yu,dthdyu,dyu2i over ju0..ju1; yv,dthdyv,dyv2i over jv0..jv1.
 * dyu2i/dyv2i are (3, j) with the three coefficients contiguous per j.
 * gw receives gridweighting(1:3,1:2) Fortran order (6 doubles). */
void lho_get_grid(const lho* s, double* yu, double* yv, double* dthdyu, double* dthdyv,
                  double* dyu2i, double* dyv2i, double* gw);

/* Canopy mask, per processed plane: planes_u[nibu_planes] (global j), mask_u[p*ngz*ngx]
 * (1 = solid point), same for v. Either pointer may be NULL. */
void lho_get_ib(const lho* s, int32_t* planes_u, uint8_t* mask_u, int32_t* planes_v, uint8_t* mask_v);

/* Fields: complex interleaved, plane-major.  u1,u3 over ju0..ju1, u2 over jv0..jv1,
 * p over jp0..jp1. */
void lho_set_fields(lho* s, const double* u1, const double* u2, const double* u3, const double* p);
void lho_get_fields(const lho* s, double* u1, double* u2, double* u3, double* p);
/* Nonlinear term of the previous substage (Nu1/Nu3 over ju0..ju1, Nu2 over jv0..jv1). */
void lho_set_nonlinear(lho* s, const double* n1, const double* n2, const double* n3);
void lho_get_nonlinear(const lho* s, double* n1, double* n2, double* n3);

/* Scalars: t, dt, mpgx, QxT.  QxT < 0 on set leaves it unchanged. */
void lho_set_scalars(lho* s, double t, double dt, double mpgx, double QxT);
void lho_get_scalars(const lho* s, double* out4);
/* flowrateIm of the current u1 (0,0) column (littleharsh.f90:412-431). */
double lho_flowrate(const lho* s);

/* One RK3 substage kRK (1..3) run up to `upto`:
 *   1 = right-hand sides assembled and divided by axz (before the canopy forcing),
 *   2 = after the canopy forcing, 3 = after the velocity solves,
 *   4 = after the flow-rate correction, 5 = the complete substage.
 * The intermediate right-hand sides can be read with lho_get_rhs. */
int  lho_substage(lho* s, int krk, int upto);
void lho_get_rhs(const lho* s, double* r1, double* r2, double* r3);
/* nsteps full RK3 steps with the current dt. Returns 0 or a negative code. */
int  lho_step(lho* s, int nsteps);

/* Diagnostics. */
double lho_divmax(lho* s);  /* max |div| over the p grid (littleharsh.f90:323-352) */
/* CFL-limited time step of the current field: CFL * min(1/max(|u|/dx+|v|/dy+|w|/dz), dtv). */
double lho_cfl_dt(lho* s, double cfl);
/* Divergence-free projection of the current field using solveP + v_corr with kRK=1. */
void lho_project(lho* s);

/* Statistics (stats.f90:1-108) accumulated from the current field.  Profiles are
 * per global y index of each grid. */
void lho_stats_accumulate(lho* s);
/* out: 13 profiles, each of length nyu (U,U2,W,W2,UV,UW,P(on u index range),P2) or nyv (V,V2,VW,wx,wx2)
 * packed as described in lh_oracle.c::lho_stats_get. Returns istat. */
int  lho_stats_get(const lho* s, double* out);
/* Conditional statistics of the wall bands (conddown/condup, stats.f90:110-253),
 * both walls summed as write_stats does; see lh_oracle.c for the layout. */
void lho_cond_accumulate(lho* s);
int  lho_cond_get(const lho* s, double* out, int32_t* dims);
void lho_spectra_accumulate(lho* s);
void lho_spectra_get(const lho* s, double* spU, double* spV, double* spW, double* spUV, double* spP);

/* Building blocks exposed for the self-pinning tests. */
/* Complex DFT in place, length n (factors 2,3,4 only), sign -1 forward, +1 inverse, unnormalised. */
int  lho_fft_c2c(int n, int sign, double* data);
/* rft (rft_buff.f:24-86): forward x (n real) -> c (n+2 reals, packed, 1/n); inverse c -> x. */
int  lho_rft(int n, int iopt, double* c);
/* Plane transforms with 3/2 padding/truncation. */
void lho_plane_to_phys(const lho* s, const double* spec, double* phys);
void lho_plane_to_spec(const lho* s, const double* phys, double* spec);
/* Tridiagonal LU (LU_dec) + solve (LUsolU) for one real right-hand side. */
void lho_tridiag_solve(int n, const double* a1, const double* a2, const double* a3, double* x);

#ifdef __cplusplus
}
#endif
#endif
