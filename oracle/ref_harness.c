/*
 * ref_harness.c -- a few lines of glue that let tests call the reference's
 * own FSM (mpi_openacc/src/phi3D_fsm.c, compiled unmodified from the
 * reference tree by oracle/Makefile) on a caller-owned halo-padded field.
 * Test infrastructure only; built into oracle/_ref/ and never shipped.
 *
 * The Phi struct is the reference's (mpi_openacc/src/phi3D.h:45-54), taken
 * from its header through the include path.
 */
#include "phi3D.h"
#include "phi3D_fsm.h"

/* Run ordering sn (1..8) of the reference solver: runFSM (phi3D_fsm.c:67). */
void ref_sweep(int nx, int ny, int nz, double dx, double dy, double dz, double *dist, int sn)
{
  Phi pf;
  pf.x = nx;
  pf.y = ny;
  pf.z = nz;
  pf.dx = dx;
  pf.dy = dy;
  pf.dz = dz;
  pf.distance = dist;
  pf.F = SPEED;
  runFSM(&pf, sn);
}
