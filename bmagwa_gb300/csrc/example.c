/* example.c -- the whole run of `bmagwa INIFILE` through the C ABI of
 * libbmg (include/bmg.h): options and PLINK data as the reference reads
 * them, one context for all chains, the reference's trace files written.
 * Build: cc -Iinclude example.c -Lbmagwa_gb300/_build -lbmg */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "bmg.h"

int main(int argc, char** argv)
{
  if (argc != 2) {
    fprintf(stderr, "usage: %s INIFILE\n", argv[0]);
    return 1;
  }
  bmg_options o;
  uint32_t seeds[64];
  char err[256];
  if (bmg_options_from_ini(argv[1], &o, seeds, 64, err, sizeof err) != BMG_OK) {
    fprintf(stderr, "%s\n", err);
    return 1;
  }
  uint8_t* bed = malloc(o.m_g * ((o.n + 3) / 4));
  double* y = malloc(o.n * sizeof(double));
  double* e = o.m_e ? malloc(o.n * o.m_e * sizeof(double)) : NULL;
  if (bmg_read_plink(&o, bed, y, e, err, sizeof err) != BMG_OK) {
    fprintf(stderr, "%s\n", err);
    return 1;
  }
  o.write_files = 1;
  bmg_ctx* ctx = NULL;
  if (bmg_create(&o, &ctx) != BMG_OK) {
    fprintf(stderr, "%s\n", bmg_last_error(NULL));
    return 1;
  }
  bmg_status st = bmg_load_bed(ctx, bed, o.n, o.m_g);
  if (st == BMG_OK) st = bmg_set_phenotypes(ctx, y, NULL, 1);
  if (st == BMG_OK) st = bmg_set_covariates(ctx, e, o.m_e);
  if (st == BMG_OK) st = bmg_precompute(ctx);
  if (st == BMG_OK) st = bmg_run(ctx, o.do_n_iter, NULL); /* or a bmg_trace_sink for in-memory traces */
  if (st == BMG_OK) st = bmg_finish(ctx);                 /* _rao.dat, _samplerstats.txt, _prior.txt */
  if (st != BMG_OK) fprintf(stderr, "%s: %s\n", bmg_status_string(st), bmg_last_error(ctx));
  bmg_destroy(ctx);
  free(bed);
  free(y);
  free(e);
  return st == BMG_OK ? 0 : 1;
}
