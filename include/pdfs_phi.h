/*
 * pdfs_phi.h -- reference-compatible surface of libpdfs: the Phi field model,
 * the run_fsm entry point, the VTI reader/writer and the whole distance-field
 * pipeline of the reference's CUDA program, on the GPU.
 *
 * pdfs_phi has the memory layout of the reference's Phi
 * (single_gpu_cuda/src/phi3D.h:45-55), so the reference's own phi3D.c /
 * main.c can link against run_fsm() below unchanged.
 */
#ifndef PDFS_PHI_H
#define PDFS_PHI_H

#include "pdfs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Layout-identical to the reference's Phi (single_gpu_cuda/src/phi3D.h:45-55). */
typedef struct {
  int x, y, z;       /* interior nodes per axis                                */
  double dx, dy, dz; /* node spacings                                          */
  int *location;     /* halo-padded flags: 1 = inside, -1 = halo/border       */
  double *distance;  /* halo-padded distances, x fastest                      */
  double F;          /* speed of propagation (1)                              */
} pdfs_phi;

/* Reference defaults (single_gpu_cuda/src/phi3D.h:37-40). */
#define PDFS_BORDER_LOCATION (-1)
#define PDFS_INTERIOR_DISTANCE 90000.0

/* Drop-in for run_fsm(Phi *, int) (single_gpu_cuda/src/phi3D_fsm.h:69-71,
 * phi3D_fsm.cu:64-106): `iterations` rounds of the 8 orderings on the GPU,
 * in place on pf->distance, in the reference's FP64 arithmetic, then prints
 * "Parallel FSM time: %f s." like the reference.  The reference returns
 * nothing and exits on CUDA errors; this one prints the error and leaves the
 * field untouched instead of exiting. */
void run_fsm(pdfs_phi *pf, int iterations);

/* Reads a VTI file in the layout the reference's reader expects
 * (single_gpu_cuda/src/vti_parser.c:85-180): the ImageData header line, then
 * after the first 6 lines the interior `location` ints, 2 more lines, the
 * interior `distance` doubles.  Allocates location/distance with malloc and
 * fills the one-node halo with PDFS_BORDER_LOCATION / +inf.  Returns PDFS_OK
 * or PDFS_ERR_IO / PDFS_ERR_INVALID / PDFS_ERR_OOM. */
int pdfs_vti_read(const char *path, pdfs_phi *pf);

/* Writes pf->distance (the whole halo-padded grid) in the reference writer's
 * format (single_gpu_cuda/src/file_writer.c:152-190), byte for byte. */
int pdfs_vti_write(const char *path, const pdfs_phi *pf);

/* Frees what pdfs_vti_read allocated. */
void pdfs_phi_free(pdfs_phi *pf);

/* The reference's calc_dist_field (single_gpu_cuda/src/phi3D.c:107-126) on
 * the GPU: pre-pass (0 -> 90000), the FSM solve, inside -> -1, halo <- inner
 * face.  rounds > 0 runs exactly that many rounds of 8 orderings (the
 * reference runs 1); rounds == 0 iterates to convergence under *o (NULL =
 * defaults).  Returns a status code. */
int pdfs_calc_dist_field(pdfs_phi *pf, int rounds, const pdfs_opts *o, pdfs_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* PDFS_PHI_H */
