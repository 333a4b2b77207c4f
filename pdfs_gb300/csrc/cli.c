/*
 * cli.c -- the PDFS command line: `PDFS <file.vti> <prefix> [options]`.
 *
 * Same invocation, console report and output file as the reference's CUDA
 * program (single_gpu_cuda/src/main.c:56-106): reads <file.vti>, computes the
 * distance field and writes <prefix>_distfield.vti.  By default it runs one
 * round of the 8 orderings, as the reference does (phi3D.c:118); options:
 *   --rounds N     run N rounds instead
 *   --converge     iterate until a sweep changes nothing (or <= --tol)
 *   --tol T        convergence tolerance on the max change (FP64)
 *   --fp32         FP32 sweeps;   --polish   FP32 sweeps + FP64 polish
 *   --fast         shifted-form FP64 arithmetic instead of the reference's
 *   --mixed        FP64 field with FP32 increments (with --polish: the fast
 *                  polish; set --tol to at least 1e-6 of the spacing)
 *   --pair         the same with an FP32-pair field (no FP64 instructions)
 *   --sched S      block scheduler: none, change or learned
 *   --device D     CUDA device
 * Exit status 0 on success, 1 on any error (message on stderr).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pdfs_phi.h"

static int usage(const char *argv0)
{
  printf("Usage: %s <file.vti> <prefix> [--rounds N | --converge] [--tol T] [--fp32 | --polish] "
         "[--fast | --mixed | --pair] [--sched none|change|learned] [--device D]\n",
         argv0);
  return 1;
}

int main(int argc, char *argv[])
{
  if (argc < 3) return usage(argv[0]);
  const char *in = argv[1], *prefix = argv[2];
  int rounds = 1;
  pdfs_opts o;
  pdfs_default_opts(&o);
  for (int i = 3; i < argc; i++) {
    if (!strcmp(argv[i], "--rounds") && i + 1 < argc) {
      rounds = atoi(argv[++i]);
      if (rounds < 1) return usage(argv[0]);
    } else if (!strcmp(argv[i], "--converge")) {
      rounds = 0;
    } else if (!strcmp(argv[i], "--tol") && i + 1 < argc) {
      o.tol = atof(argv[++i]);
    } else if (!strcmp(argv[i], "--fp32")) {
      o.precision = PDFS_PREC_FP32;
    } else if (!strcmp(argv[i], "--polish")) {
      o.precision = PDFS_PREC_FP32_POLISH64;
      if (o.arith == PDFS_ARITH_REFERENCE) o.arith = PDFS_ARITH_FAST;
    } else if (!strcmp(argv[i], "--fast")) {
      o.arith = PDFS_ARITH_FAST;
    } else if (!strcmp(argv[i], "--mixed")) {
      o.arith = PDFS_ARITH_MIXED;
    } else if (!strcmp(argv[i], "--pair")) {
      o.arith = PDFS_ARITH_PAIR;
    } else if (!strcmp(argv[i], "--sched") && i + 1 < argc) {
      const char *v = argv[++i];
      if (!strcmp(v, "none"))
        o.scheduler = PDFS_SCHED_NONE;
      else if (!strcmp(v, "change"))
        o.scheduler = PDFS_SCHED_CHANGE;
      else if (!strcmp(v, "learned"))
        o.scheduler = PDFS_SCHED_LEARNED;
      else
        return usage(argv[0]);
    } else if (!strcmp(argv[i], "--device") && i + 1 < argc) {
      o.device = atoi(argv[++i]);
    } else {
      return usage(argv[0]);
    }
  }
  if (o.precision == PDFS_PREC_FP32_POLISH64) rounds = 0;  /* the polish is a convergence loop */

  pdfs_phi pf;
  int s = pdfs_vti_read(in, &pf);
  if (s == PDFS_ERR_IO) {
    printf("Unable to read file \"%s\"!\n", in);
    return 1;
  }
  if (s != PDFS_OK) {
    fprintf(stderr, "PDFS: %s\n", pdfs_status_string(s));
    return 1;
  }
  printf("Dimensions:\n");
  printf("x: %d\tdx: %f\n", pf.x, pf.dx);
  printf("y: %d\tdy: %f\n", pf.y, pf.dy);
  printf("z: %d\tdz: %f\n", pf.z, pf.dz);

  pdfs_stats st;
  s = pdfs_calc_dist_field(&pf, rounds, &o, &st);
  if (s != PDFS_OK) {
    fprintf(stderr, "PDFS: %s (%d)\n", pdfs_status_string(s), s);
    pdfs_phi_free(&pf);
    return 1;
  }
  printf("Parallel FSM time: %f s.\n", (st.ms_fp32 + st.ms_fp64) / 1000.0);

  size_t len = strlen(prefix) + 32;
  char *out = (char *) malloc(len);
  if (!out) {
    pdfs_phi_free(&pf);
    return 1;
  }
  snprintf(out, len, "%s_distfield.vti", prefix);
  s = pdfs_vti_write(out, &pf);
  if (s == PDFS_OK) printf("VTI file created: %s\n", out);
  else fprintf(stderr, "PDFS: cannot write %s\n", out);
  free(out);
  pdfs_phi_free(&pf);
  return s == PDFS_OK ? 0 : 1;
}
