/*
 * lh_driver.c -- a C host driver for the GB300 RK3 step, in the order of the
 * reference's main program (littleharsh.f90:63-208) for users without a
 * Fortran compiler.  It calls only the C ABI of include/littleharsh.h.
 *
 *   lh_driver <input.in> [--steps N] [--out DIR] [--name NAME] [--mixed]
 *
 * start (start.f90:36-652)      lh_read_input, lh_setup_grid, lh_setup_canopy, lh_init
 * getini (start.f90:1488-1594)  flag_init 1/2: the restart files <dirin>/u1<name> ... read as read_in reads
 *                               them (name = fnameimb without its leading "u1"); flag_init 3: the parabolic
 *                               profile of mblock_ini_parabolic_profile (start.f90:1644-1784).  flag_init 1 and 3
 *                               start at t = 0, 2 at the file's time; QxT is the start field's flow rate
 *                               (start.f90:1515-1518); mpgx is input.in's.
 * main loop (littleharsh.f90:161-201)
 *                               lh_rk3_step until t >= maxt (or N steps with --steps), dt from the CFL number
 *                               (re-evaluated every nwrite steps), max |div| checked against maxerr every nwrite
 *                               steps (error, littleharsh.f90:323-352), a progress line every nwrite steps
 * finalize (littleharsh.f90:354-410)
 *                               the fields written as restart files <DIR>/u1<NAME> ... (default DIR = dirout,
 *                               NAME = _final.dat) and the accumulated statistics and spectra of the run
 *                               (sampled every nwrite steps) to <DIR>/stats<NAME> and <DIR>/sp*_<NAME>.
 * Exit status 0, or 1 with the library's reason on stderr.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "littleharsh.h"

static int check(int rc, lh_handle* h, const char* what) {
  if (rc != LH_OK) fprintf(stderr, "lh_driver: %s failed (%d): %s\n", what, rc, lh_last_error(h));
  return rc != LH_OK;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s <input.in> [--steps N] [--out DIR] [--name NAME] [--mixed]\n", argv[0]);
    return 2;
  }
  const char* inpath = argv[1];
  long max_steps = -1;
  const char* outdir = NULL;
  const char* outname = "_final.dat";
  int precision = LH_PREC_FP64;
  for (int a = 2; a < argc; ++a) {
    if (!strcmp(argv[a], "--steps") && a + 1 < argc) max_steps = atol(argv[++a]);
    else if (!strcmp(argv[a], "--out") && a + 1 < argc) outdir = argv[++a];
    else if (!strcmp(argv[a], "--name") && a + 1 < argc) outname = argv[++a];
    else if (!strcmp(argv[a], "--mixed")) precision = LH_PREC_MIXED;
    else {
      fprintf(stderr, "lh_driver: unknown argument %s\n", argv[a]);
      return 2;
    }
  }

  /* start: input.in, the y grid and the canopy lists */
  lh_input in;
  lh_params prm;
  memset(&prm, 0, sizeof prm);
  if (check(lh_read_input(inpath, &in), NULL, "lh_read_input")) return 1;
  const int dsty = in.dsty > 0 ? in.dsty : 0;
  const int nyu = in.ny + 2 * dsty + 1, nyv = in.ny + 2 * dsty;
  double* yu = calloc(nyu, sizeof(double));
  double* yv = calloc(nyv, sizeof(double));
  double* dthdyu = calloc(nyu, sizeof(double));
  double* dthdyv = calloc(nyv, sizeof(double));
  double* dyu2i = calloc(3 * (size_t)nyu, sizeof(double));
  double* dyv2i = calloc(3 * (size_t)nyv, sizeof(double));
  if (check(lh_setup_grid(&in, &prm, yu, yv, dthdyu, dthdyv, dyu2i, dyv2i), NULL, "lh_setup_grid")) return 1;
  int32_t nlu = 0, nlv = 0;
  if (check(lh_setup_canopy(&in, &prm, NULL, &nlu, NULL, &nlv), NULL, "lh_setup_canopy")) return 1;
  int32_t* lu = calloc(3 * (size_t)(nlu > 0 ? nlu : 1), sizeof(int32_t));
  int32_t* lv = calloc(3 * (size_t)(nlv > 0 ? nlv : 1), sizeof(int32_t));
  if ((nlu || nlv) && check(lh_setup_canopy(&in, &prm, lu, &nlu, lv, &nlv), NULL, "lh_setup_canopy")) return 1;
  prm.precision = precision;
  lh_handle* h = NULL;
  if (check(lh_init(&prm, yu, yv, dthdyu, dthdyv, dyu2i, dyv2i, lu, nlu, lv, nlv, &h), NULL, "lh_init")) return 1;
  int32_t sz[12];
  if (check(lh_get_sizes(h, sz), h, "lh_get_sizes")) return 1;
  const size_t plane = (size_t)sz[0] * sz[1];
  const int nyp = sz[6];

  /* getini */
  double t = 0.0;
  int32_t iter = 0;
  if (in.flag_init == 1 || in.flag_init == 2) {
    const char* name = strncmp(in.fnameimb, "u1", 2) == 0 ? in.fnameimb + 2 : in.fnameimb;
    double tf = 0.0;
    if (check(lh_read_restart(h, in.dirin, name, &tf, &iter), h, "lh_read_restart")) return 1;
    if (in.flag_init == 1) {
      t = 0.0;
      iter = 0;
    } else {
      t = tf;
    }
  } else if (in.flag_init == 3) {
    /* mblock_ini_parabolic_profile: the (0,0) modes of every level */
    double* u1 = calloc(2 * plane * nyu, sizeof(double));
    double* u2 = calloc(2 * plane * nyv, sizeof(double));
    double* u3 = calloc(2 * plane * nyu, sizeof(double));
    double* p = calloc(2 * plane * nyp, sizeof(double));
    for (int j = 0; j < nyu; ++j) {
      u1[2 * plane * j] = 0.5 * in.Re * in.mpgx * (yu[j] * yu[j] - 1.0);
      u3[2 * plane * j] = 1e-5;
    }
    for (int j = 0; j < nyv; ++j) u2[2 * plane * j] = 1e-6;
    for (int j = 0; j < nyp; ++j) p[2 * plane * j] = 1.0;
    if (check(lh_set_fields(h, u1, u2, u3, p, LH_LAYOUT_PLANES), h, "lh_set_fields")) return 1;
    free(u1); free(u2); free(u3); free(p);
  } else {
    fprintf(stderr, "lh_driver: flag_init %d: initial conditions not implemented (as in getini)\n", in.flag_init);
    return 1;
  }
  double dt = 0.0;
  if (check(lh_cfl_dt(h, in.CFL, &dt), h, "lh_cfl_dt")) return 1;
  if (check(lh_set_time(h, t, dt, in.mpgx, -1.0), h, "lh_set_time")) return 1;
  const int nwrite = in.nwrite > 0 ? in.nwrite : 1;
  if (check(lh_set_monitor(h, in.maxerr, nwrite), h, "lh_set_monitor")) return 1;

  /* main loop (littleharsh.f90:161-201), nwrite steps at a time */
  long done = 0;
  while (t < in.maxt && (max_steps < 0 || done < max_steps)) {
    long n = nwrite;
    if (max_steps >= 0 && max_steps - done < n) n = max_steps - done;
    if (check(lh_rk3_step(h, (int32_t)n), h, "lh_rk3_step")) return 1;
    done += n;
    iter += (int32_t)n;
    double tm[5], dm = 0.0;
    if (check(lh_get_time(h, tm), h, "lh_get_time") || check(lh_get_monitor(h, &dm, NULL), h, "lh_get_monitor"))
      return 1;
    t = tm[0];
    printf("iter %8d  t %.6e  dt %.4e  mpgx %.6e  Qx %.10e  max|div| %.3e\n", iter, t, tm[1], tm[2], tm[4], dm);
    if (check(lh_stats_accumulate(h), h, "lh_stats_accumulate") || check(lh_cond_accumulate(h), h, "lh_cond_accumulate") ||
        check(lh_spectra_accumulate(h), h, "lh_spectra_accumulate"))
      return 1;
    double dtn = 0.0;
    if (check(lh_cfl_dt(h, in.CFL, &dtn), h, "lh_cfl_dt")) return 1;
    if (check(lh_set_time(h, t, dtn, tm[2], -1.0), h, "lh_set_time")) return 1;
  }

  /* finalize: restart files, statistics and spectra */
  const char* dir = outdir ? outdir : in.dirout;
  char path[1024];
  snprintf(path, sizeof path, "%s/stats%s", dir, outname);
  if (check(lh_write_restart(h, &prm, yu, yv, dir, outname, iter), h, "lh_write_restart")) return 1;
  if (check(lh_write_stats(h, &prm, yu, yv, dthdyu, dthdyv, path, iter), h, "lh_write_stats")) return 1;
  if (check(lh_write_spectra(h, &prm, yu, yv, dthdyu, dthdyv, dir, outname, iter), h, "lh_write_spectra")) return 1;
  double dm = 0.0;
  if (check(lh_divmax(h, &dm), h, "lh_divmax")) return 1;
  printf("done: %ld steps, t %.6e, max|div| %.3e\n", done, t, dm);
  lh_free(h);
  free(yu); free(yv); free(dthdyu); free(dthdyv); free(dyu2i); free(dyv2i); free(lu); free(lv);
  return 0;
}
