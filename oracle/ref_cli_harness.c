/*
 * ref_cli_harness.c -- lets the reference's own CUDA-program sources
 * (single_gpu_cuda/src/main.c, phi3D.c, vti_parser.c, file_writer.c) build
 * into a CPU binary: it supplies run_fsm(Phi *, int) (the reference's CUDA
 * entry, single_gpu_cuda/src/phi3D_fsm.h:69-71) on top of the reference's
 * CPU sweep runFSM (mpi_openacc/src/phi3D_fsm.c:67).  Test infrastructure:
 * built into oracle/_ref/ only, to produce golden files with the reference's
 * reader, pre/post passes and writer.
 */
#include "phi3D.h" /* single_gpu_cuda/src/phi3D.h: Phi with a location array */

/* Field layout of the OpenACC program's Phi (mpi_openacc/src/phi3D.h:45-54). */
typedef struct {
  int x, y, z;
  double dx, dy, dz;
  double *distance;
  double F;
} AccPhi;

void runFSM(AccPhi *pf, int sn);

void run_fsm(Phi *pf, int iterations)
{
  AccPhi m = {pf->x, pf->y, pf->z, pf->dx, pf->dy, pf->dz, pf->distance, pf->F};
  for (int r = 0; r < iterations; r++)
    for (int sn = 1; sn <= 8; sn++) runFSM(&m, sn);
}
