/*
 * littleharsh.h -- C ABI of the GB300 RK3 time step for Littleharsh.
 *
 * The reference advances its channel-over-canopy DNS with plain Fortran calls
 * from the main loop (littleharsh.f90:164-190):
 *     RHS0_u1/u2/u3, nonlinear, solveU/solveV/solveU, meanflow_ctU, solveP, v_corr
 * on fields held in the module `declaration` (declaration.f90:133-135,
 * type(cfield), complex(8) f(j, column)).  This header replaces that whole
 * loop body with one call, lh_rk3_step, on device-resident fields owned by a
 * handle.  The Fortran driver (start.f90 setup, input.in, output) keeps its
 * role: it computes the y grid and the canopy point lists exactly as before
 * and hands them to lh_init; a driver without a Fortran compiler can call the
 * host helpers at the end of this header, which restate that setup.
 *
 * Conventions (all entry points):
 *   - return 0 on success or a negative LH_E* code; lh_last_error(handle)
 *     gives a one-line reason (lh_last_error(NULL) for failures before a
 *     handle exists);
 *   - the caller owns every host buffer; the handle owns all device memory;
 *   - calls on one handle are not thread-safe; separate handles are
 *     independent; each handle works on the CUDA device that was current when
 *     lh_init ran and on the stream given in lh_params (0 = legacy default);
 *   - complex values are interleaved (re, im) doubles, the ABI of Fortran
 *     complex(8), C double _Complex and cuDoubleComplex.
 *
 * Field layouts (layout argument):
 *   LH_LAYOUT_PLANES   [j][kk][i]: plane-major, i = 0..N1/2 fastest, then
 *                      kk = 0..N2-1 in FFT order (kz = bet*kk for kk < N2/2,
 *                      bet*(kk-N2) otherwise), then the y index j of the
 *                      field's own grid.  This is the device layout.
 *   LH_LAYOUT_COLUMNS  the reference's cfield f(j, column) for the single
 *                      band of long columns (proc_lims_columns, start.f90:
 *                      1092-1105, one process): j fastest, column =
 *                      kk*(N1/2+1) + i.  The conversion is an in-HBM
 *                      transpose on the device.
 * Grids: u and w on the u grid j = N(4,0)..N(4,3)+1 (centres with ghosts),
 * v on the v grid j = N(3,0)..N(3,3)+1 (faces, walls included), p on
 * j = N(4,0)+1..N(4,3) (jlim, start.f90:1155-1174).
 */
#ifndef LITTLEHARSH_H
#define LITTLEHARSH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: lh_stats_flush fills rows 11-12 (omega_x) and lh_cond_flush returns 13 blocks */
#define LH_ABI_VERSION 2

enum {
  LH_OK = 0,
  LH_EINVAL = -1,       /* bad argument, shape or parameter */
  LH_EUNSUPPORTED = -2, /* valid for the reference but not built here (e.g. two x/z resolutions) */
  LH_EFFT = -3,         /* a transform length does not factor into 2, 3 and 4 */
  LH_ECUDA = -4,        /* CUDA runtime error */
  LH_ENOMEM = -5,       /* device allocation failed */
  LH_ESTATE = -6,       /* call out of order (e.g. step before fields or dt) */
  LH_ENUMERIC = -7      /* non-finite value detected */
};

enum { LH_LAYOUT_PLANES = 0, LH_LAYOUT_COLUMNS = 1 };
enum { LH_PREC_FP64 = 0, LH_PREC_MIXED = 1 };

typedef struct lh_handle lh_handle;
typedef struct lh_ensemble lh_ensemble;

/* Everything lh_init needs besides the grid arrays.  Integer arrays follow
 * the reference's Fortran storage: N(1:4,0:nband+1) is N[(band)*4 + row-1]. */
typedef struct lh_params {
  int32_t abi_version;     /* LH_ABI_VERSION */
  int32_t N[20];           /* N(1:4,0:4)    (declaration.f90:25, set in start.f90/y_grid_canopy.f90) */
  int32_t Ngal[20];        /* Ngal(1:4,0:4) */
  int32_t nn;              /* nn after y_grid_canopy (= input ny - 2) */
  int32_t flag_ctpress;    /* 0: constant flow rate (meanflow_ctU), 1: constant pressure gradient */
  int32_t geometry_type;   /* 0 smooth, 3 canopies (only 3 has a forcing list) */
  int32_t dsty;            /* canopy points in y, as in input.in */
  double Re, alp, bet;
  double ddthetavi;        /* 1/dtheta from y_grid_canopy (1 in the reference) */
  double gridweighting[6]; /* gridweighting(1:3,1:2), Fortran order (start.f90:497-503) */
  int32_t precision;       /* LH_PREC_FP64 or LH_PREC_MIXED */
  int32_t ntilex, ntilez;  /* canopy tiles in x and z (input.in), for the conditional statistics */
  int32_t reserved;
  void* stream;            /* cudaStream_t, NULL = default stream */
} lh_params;

/* Create a solver.  Replaces the device-relevant half of `start`
 * (start.f90:36-652): wavenumbers (def_k :655-704), RK3 coefficients
 * (:413-427), the pressure LU (LU_buildP :628-630) and the canopy forcing
 * lists distributed by getbounds (:706-998).
 *   yu, dthdyu:  N(4,0)..N(4,3)+1      yv, dthdyv: N(3,0)..N(3,3)+1
 *   dyu2i:       (3, N(4,0):N(4,3)+1)  dyv2i:      (3, N(3,0):N(3,3)+1)
 *   list_u/list_v: (3, n) Fortran order (i, k, j), 1-based physical i,k and
 *   global j: list_ib(:,:,ugrid) and list_ib(:,:,vgrid) of both canopies as
 *   boundary_canopies builds them (geom_sym_canopy.f90:97-234).  Points on
 *   planes outside the ranges getbounds hands out are dropped, as there. */
int lh_init(const lh_params* prm, const double* yu, const double* yv, const double* dthdyu,
            const double* dthdyv, const double* dyu2i, const double* dyv2i, const int32_t* list_u,
            int32_t nlist_u, const int32_t* list_v, int32_t nlist_v, lh_handle** out);

/* Release the handle and its device memory (part of `finalize`, littleharsh.f90:354-410). */
void lh_free(lh_handle* h);

/* Reason for the last failure on h (or of the last failed lh_init when h is NULL). */
const char* lh_last_error(const lh_handle* h);

/* Sizes: out[0..11] = nkx, nz, ngx, ngz, nyu, nyv, nyp, ju0, jv0, jp0, n_ib_planes_u, n_ib_planes_v. */
int lh_get_sizes(const lh_handle* h, int32_t* out12);

/* Upload / download u1, u2, u3, p (any may be NULL).  Uploading u1 with
 * flag_ctpress = 0 sets the target flow rate QxT from its (0,0) column, as
 * getini does (start.f90:1515-1518). */
int lh_set_fields(lh_handle* h, const double* u1, const double* u2, const double* u3, const double* p,
                  int32_t layout);
int lh_get_fields(lh_handle* h, double* u1, double* u2, double* u3, double* p, int32_t layout);

/* Nonlinear term of the previous substage (Nu1, Nu2, Nu3), same layouts. */
int lh_set_nonlinear(lh_handle* h, const double* n1, const double* n2, const double* n3, int32_t layout);
int lh_get_nonlinear(lh_handle* h, double* n1, double* n2, double* n3, int32_t layout);

/* Scalars t, dt, mpgx; QxT < 0 keeps the current target flow rate. */
int lh_set_time(lh_handle* h, double t, double dt, double mpgx, double QxT);
/* out[0..4] = t, dt, mpgx, QxT, Qx (flowrateIm of the current u1). */
int lh_get_time(lh_handle* h, double* out5);

/* Advance nsteps full RK3 steps (the body of the main loop,
 * littleharsh.f90:164-199) with the current dt.  The device work of one step
 * is captured once into a CUDA graph and replayed.  Returns LH_ENUMERIC when
 * a NaN or an infinity reached the fields (the pressure solve, which sees the
 * divergence of every column, flags it on the device at no extra pass; the
 * flag is read once per call, or once per monitor block), or when the
 * monitor's max |div| exceeds maxerr; lh_last_error names the steps.  The
 * fields are left as they are for inspection; uploading fields clears the
 * flag. */
int lh_rk3_step(lh_handle* h, int32_t nsteps);

/* Step monitor.  The reference computes max |div| after each substage's
 * correction (v_corr, littleharsh.f90:933-935) and reports it through
 * `error` (littleharsh.f90:323-352) against input.in's maxerr
 * (start.f90:160,430).  With every > 0, lh_rk3_step runs its steps in blocks
 * of `every`, and after each block computes max |div| on the device and
 * returns LH_ENUMERIC if it exceeds maxerr; every = 0 (the default) turns the
 * monitor off.  The monitor's kernels run outside the timed graph launches
 * (lh_last_step_ms excludes them). */
int lh_set_monitor(lh_handle* h, double maxerr, int32_t every);
/* The last max |div| the monitor measured (-1 before its first block) and the
 * device's sticky error bits (1 = non-finite value).  Either pointer may be
 * NULL.  No counterpart in the reference beyond `error`'s err. */
int lh_get_monitor(lh_handle* h, double* divmax, int32_t* err_bits);

/* FP64 FMA throughput of the current device in TFLOP/s, measured by a probe
 * kernel of this library (eight independent FMA chains per thread, best of
 * three CUDA-event-timed launches); the denominator of the FP64 roofline the
 * benchmark reports.  No counterpart in the reference. */
int lh_fp64_peak(double* tflops);

/* One substage kRK (1..3) up to `upto` (1 right-hand sides divided by axz,
 * 2 after the canopy forcing, 3 after the velocity solves, 4 after the
 * flow-rate correction, 5 complete); lh_get_rhs reads the right-hand sides. */
int lh_substage(lh_handle* h, int32_t krk, int32_t upto);
int lh_get_rhs(lh_handle* h, double* r1, double* r2, double* r3, int32_t layout);

/* max |div u| over the p grid (error, littleharsh.f90:323-352). */
int lh_divmax(lh_handle* h, double* out);
/* CFL time step of the current field: cfl * min(1/max(|u|/dx+|v|/dy+|w|/dz), dtv). */
int lh_cfl_dt(lh_handle* h, double cfl, double* dt_out);
/* Divergence-free projection of the current velocity (solveP + v_corr with kRK = 1). */
int lh_project(lh_handle* h);

/* Spectra (spectra.f90:1-56): accumulate |u|^2, |v|^2, |w|^2, Re(u conj v_c),
 * |p|^2 per (j, column) on the device in FP64; flush returns the sums in
 * LH_LAYOUT_PLANES order (real, nyu/nyv/nyu/nyu/nyp planes) and the count. */
int lh_spectra_accumulate(lh_handle* h);
int lh_spectra_flush(lh_handle* h, double* spU, double* spV, double* spW, double* spUV, double* spP,
                     int32_t* count, int32_t reset);

/* Plane statistics (stats.f90:1-108), FP64 sums over the physical planes of
 * each level: out is 13 x max(nyu, nyv): Um U2m Vm V2m Wm W2m Pm P2m UVm UWm
 * VWm wxm wx2m.  Rows on the v or p grid use their first nyv / nyp entries.
 * UVm pairs u with v interpolated to the centres, VWm v with w interpolated to
 * the faces (both zero on ghost centres / wall faces).  wxm, wx2m are the
 * streamwise vorticity omega_x = dw/dy - dv/dz on every face, the y-difference
 * of w across the face with the pressure gradient's metric dthdyv
 * (littleharsh.f90:685) minus i kz v (the routine that fills the reference's
 * wx, in FOU3D.f90, is missing).  Every row sums the whole plane; the
 * reference's wx loop covers only i <= N(1), k <= N(2) of its Ngal-sized wx
 * array (stats.f90:53-58), bounds left from an earlier N-grid allocation
 * (start.f90:637-638).  The sums are formed from the spectral coefficients
 * (Parseval on the 3/2 grid), equal to the physical sums up to rounding.
 * Call between steps: it reuses the right-hand-side scratch. */
int lh_stats_accumulate(lh_handle* h);
int lh_stats_flush(lh_handle* h, double* out, int32_t* count, int32_t reset);

/* Conditional statistics of the wall bands (conddown1/2 and condup1/2,
 * stats.f90:110-253): sums over the ntilex x ntilez canopy tiles at each
 * in-tile point (dnx = Ngalx/ntilex by dnz = Ngalz/ntilez), for the planes of
 * the bottom band counted from its wall plus those of the top band counted
 * from the top wall with v's sign flipped (write_stats sums the two,
 * stats.f90:473-512), accumulated in FP64 from physical planes.  dims[0..4] =
 * nju, njv, njp, dnx, dnz (nju = N(4,1)-N(4,0)+1, njv = N(3,1)-N(3,0)+1,
 * njp = N(4,1)-N(4,0)-1; all 0 without canopies).  out: 13 blocks
 * [j1][kin][i] (i fastest): UmC U2mC WmC W2mC UVmC UWmC (nju planes), VmC
 * V2mC VWmC (njv), PmC P2mC (njp), wxmC wx2mC (njv; omega_x keeps its sign on
 * the top wall, as condup1 is called with xsign = 1 for wx, stats.f90:102).
 * Call between steps. */
int lh_cond_accumulate(lh_handle* h);
int lh_cond_flush(lh_handle* h, double* out, int32_t* dims5, int32_t* count, int32_t reset);

/* Ensembles of independent replicas (uneven grids and geometries allowed) on
 * one device: lh_ensemble_step advances every member by nsteps RK3 steps with
 * one CUDA-graph launch per step.  Members keep their own state and can still
 * be used alone.  ms (may be NULL) receives the device time.  No counterpart
 * in the reference (one simulation per MPI job), whose per-replica loop is
 * the main loop itself (littleharsh.f90:161-201).
 * Modes (lh_ensemble_set_mode):
 *   LH_ENS_STREAMS (default)  the graph forks into each member's stream,
 *     each member launching its own kernels, so the members' kernels overlap.
 *   LH_ENS_BATCHED  one launch per kernel kind and slot of the substage
 *     (each band's z-inverse, product pass and z-forward, assembly, canopy
 *     forcing, Thomas sweeps, flow rate, pressure solve) for every grid class
 *     (members with the same grid) and shared-memory size, covering the
 *     blocks of all its members, with the members' arguments in the launch's
 *     kernel parameter (up to 32 members per launch); the classes' launches
 *     run on streams of their own.  The launches per step do not grow with
 *     the member count.  Needs members of one precision; otherwise the
 *     streams mode is used.
 * Either way each member's arithmetic is that of its own lh_rk3_step, bit for
 * bit.  lh_ensemble_info reports the mode of the captured graph and its
 * kernel launches per step. */
enum { LH_ENS_STREAMS = 0, LH_ENS_BATCHED = 1 };
int lh_ensemble_create(lh_handle* const* members, int32_t n, lh_ensemble** out);
int lh_ensemble_set_mode(lh_ensemble* e, int32_t mode);
int lh_ensemble_step(lh_ensemble* e, int32_t nsteps, double* ms);
int lh_ensemble_info(const lh_ensemble* e, int32_t* mode_used, int32_t* launches_per_step);
const char* lh_ensemble_last_error(const lh_ensemble* e);
void lh_ensemble_free(lh_ensemble* e);

/* Device time of the last lh_rk3_step call in milliseconds (CUDA events on
 * the handle's stream) and the number of kernels one step launches. */
int lh_last_step_ms(lh_handle* h, double* ms, int32_t* launches_per_step);

/* Advance one RK3 step launch by launch (no graph) with a CUDA event after each
 * kernel, and return the device time and launch count per kernel kind:
 * 0 z-inverse, 1 x-pass with products, 2 z-forward, 3 right-hand-side
 * assembly, 4/5/6 canopy forcing z-inverse / x-mask / z-forward, 7 velocity
 * Thomas, 8 flow-rate correction, 9 pressure solve + correction.
 * nkinds must be at least 10. */
int lh_profile_step(lh_handle* h, double* ms_by_kind, int32_t* count_by_kind, int32_t nkinds);

/* Launch-shape autotuner (no reference counterpart).  On this handle's grid
 * and precision it times, in turn, the z passes for each z tile width
 * (columns per CTA) and then for 128 and 256 threads per CTA, the product pass
 * for each number of levels per CTA, its buffer split, and its threads per CTA
 * together with (in the mixed form) one or two z rows per CTA; it keeps the
 * fastest of each and returns the tile width and the levels per CTA (either
 * pointer may be NULL; read the rest back with lh_get_launch_shapes,
 * lh_get_z_threads, lh_get_x_threads and lh_get_x_rows).  Needs fields; writes
 * only scratch, so the fields and the time are unchanged, and every choice
 * gives the same results bit for bit.  The next step is captured with the new
 * shapes. */
int lh_autotune(lh_handle* h, int32_t* tx, int32_t* chunk);

/* The launch shapes the next step uses (no reference counterpart): z tile
 * width, levels per product-pass CTA, and whether the product pass transforms
 * the face pair after the centre pairs through a smaller buffer (1) or all
 * three pairs at once (0); lh_autotune picks that by timing too.  Any pointer
 * may be NULL. */
int lh_get_launch_shapes(lh_handle* h, int32_t* tx, int32_t* chunk, int32_t* xsplit);

/* Threads per product-pass CTA the next step uses (128 or 256; no reference
 * counterpart); lh_autotune picks it by timing.  Batched ensemble launches
 * always use 256. */
int lh_get_x_threads(lh_handle* h, int32_t* threads);

/* Threads per CTA of the z passes (nonlinear term and canopy forcing) the
 * next step uses (128 or 256; no reference counterpart); lh_autotune picks it
 * by timing at the z tile width it chose.  Batched ensemble launches always
 * use 256. */
int lh_get_z_threads(lh_handle* h, int32_t* threads);

/* z rows per product-pass CTA the next step uses (no reference counterpart):
 * 2 when the mixed form runs two rows' FP32 transforms in lockstep (the same
 * arithmetic per row, so the same results), else 1; lh_autotune picks it by
 * timing.  Batched ensemble launches always use 1. */
int lh_get_x_rows(lh_handle* h, int32_t* rows);

/* Divergence-free projection (solveP + v_corr with kRK = 1, the operation of
 * lh_project) of caller-owned device arrays u1, u2, u3 (plane layout), for
 * callers that cannot allocate device memory: a Fortran driver whose fields
 * live in OpenACC or CUDA Fortran device arrays, or an application that owns
 * all GPU memory through one arena and must not call cudaMalloc mid-run.
 * No counterpart in the reference.  It needs no handle and allocates nothing:
 * its scratch (wavenumbers, metric, pressure LU, psi, p) is a 64 MiB static
 * device array that every GPU loading the library holds until exit, which
 * limits the grid to about 48 bytes x nyp x (N1/2+1) x N2 <= 64 MiB
 * (configuration 1 fits, configuration 2 does not); larger grids return
 * LH_EINVAL with the reason in lh_last_error(NULL).  prm, yu, dthdyu and
 * dthdyv are the host arrays lh_init takes, checked as lh_init checks them;
 * grids with two x/z resolutions return LH_EUNSUPPORTED.  dt only scales psi
 * (it cancels).  Every call looks up the array's device address on the
 * current device.  With lazy module loading (CUDA_MODULE_LOADING=LAZY, the
 * default) the 64 MiB is placed on a device at the first call there, not when
 * the library loads.  The call copies tables from host memory and waits for
 * its stream, so it cannot be made while that stream is capturing a graph.
 * All calls share the array: calls whose work overlaps on the GPU race.  Runs
 * on `stream` (cudaStream_t, NULL = default) of the current device and
 * returns after the projection has finished. */
int lh_project_noalloc(const lh_params* prm, const double* yu, const double* dthdyu, const double* dthdyv,
                       double* u1, double* u2, double* u3, double dt, void* stream);

/* ---------------------------------------------------------------------------
 * The reference's files.  Fortran sequential unformatted records (4-byte
 * length before and after each record).
 * ------------------------------------------------------------------------- */

/* Restart fields in the format read_in reads (start.f90:1786-2235): files
 * <dir>/u1<name>, u2<name>, u3<name>, p<name> (name = fnameimb(3:) in the
 * reference); records: header (t, Re, alp, bet, mpgx, nband, iter, 88 ints),
 * N(4,0:4), one record read_in skips (the field's y coordinates), then one
 * record per plane of the field's grid: jin, band, nx = N1+2, nz = N2, y(jin),
 * buffSR(nx, nz) -- the packed x half-spectrum of the plane's z modes.
 * prm is the block given to lh_init; yu, yv its grid arrays. */
int lh_write_restart(lh_handle* h, const lh_params* prm, const double* yu, const double* yv, const char* dir,
                     const char* name, int32_t iter);
/* Read the four files (the grid must match: LH_EUNSUPPORTED otherwise) and
 * upload them as lh_set_fields does (QxT from u1 for constant flow rate). */
int lh_read_restart(lh_handle* h, const char* dir, const char* name, double* t_out, int32_t* iter_out);
/* write_stats (stats.f90:355-410) of the accumulated plane and conditional
 * statistics to `path`; resets the accumulators as write_stats does. */
int lh_write_stats(lh_handle* h, const lh_params* prm, const double* yu, const double* yv, const double* dthdyu,
                   const double* dthdyv, const char* path, int32_t iter);
/* recvwrspec (spectra.f90:109-180): <dir>/spU_<name> ... spP_<name>, kz and
 * -kz folded and kx >= 1 doubled; resets the accumulators. */
int lh_write_spectra(lh_handle* h, const lh_params* prm, const double* yu, const double* yv, const double* dthdyu,
                     const double* dthdyv, const char* dir, const char* name, int32_t iter);

/* ---------------------------------------------------------------------------
 * Host helpers restating the setup the Fortran driver does in start.f90, for
 * drivers without a Fortran compiler.
 * ------------------------------------------------------------------------- */

/* Parsed input.in (start.f90:63-196, fixed-column FORMATs :433-436). */
typedef struct lh_input {
  double Re, alp, bet;
  int32_t ngalx1, ngalx2, ngalz1, ngalz2, ny;
  double dyq;
  int32_t ppp, flag_init;
  char fnameimb[96], dirin[96], dirout[96];
  double CFL;
  int32_t nwrite, flag_ctpress;
  double mpgx, Kib, maxerr, maxt, maxA;
  int32_t physlim_bot, physlim_top, geometry_type, ntilex, ntilez;
  double posth;
  int32_t npeakx, npeakz;
  double Lfracx, Lfracz;
  int32_t dsty, dstx, dstz;
} lh_input;

int lh_read_input(const char* path, lh_input* out);

/* y_grid_canopy (y_grid_canopy.f90:24-194) and the band bookkeeping: fills
 * prm (N, Ngal, nn, ddthetavi, gridweighting, Re, alp, bet, flag_ctpress,
 * geometry_type, dsty) and the grid arrays, whose lengths are
 * nyu = ny + 2*dsty + 1 and nyv = ny + 2*dsty. */
int lh_setup_grid(const lh_input* in, lh_params* prm, double* yu, double* yv, double* dthdyu,
                  double* dthdyv, double* dyu2i, double* dyv2i);

/* boundary_canopies (geom_sym_canopy.f90:63-234): both canopies' lists.
 * Call with list_u/list_v NULL to get the counts. */
int lh_setup_canopy(const lh_input* in, const lh_params* prm, int32_t* list_u, int32_t* nlist_u,
                    int32_t* list_v, int32_t* nlist_v);

#ifdef __cplusplus
}
#endif
#endif
