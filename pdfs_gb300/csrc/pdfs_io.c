/*
 * pdfs_io.c -- VTI reader and writer of the reference's file formats.
 *
 * The formats are the interface the reference's users have files in, so the
 * reader accepts what single_gpu_cuda/src/vti_parser.c:85-180 accepts and the
 * writer emits what single_gpu_cuda/src/file_writer.c:152-190 emits, byte for
 * byte.  The reader is more tolerant of the header's whitespace than the
 * reference's fixed sscanf format, and it checks every conversion.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pdfs_phi.h"

/* Header: ... WholeExtent="0 X 0 Y 0 Z" ... Spacing="dx dy dz" ... ; the
 * interior node counts are X+1, Y+1, Z+1 (single_gpu_cuda/src/phi3D.c:57-62). */
static int parse_header(const char *line, double d[6])
{
  const char *p = strstr(line, "WholeExtent=\"");
  const char *q = strstr(line, "Spacing=\"");
  if (!p || !q) return 0;
  if (sscanf(p + 13, "0 %lf 0 %lf 0 %lf", &d[0], &d[1], &d[2]) != 3) return 0;
  if (sscanf(q + 9, "%lf %lf %lf", &d[3], &d[4], &d[5]) != 3) return 0;
  return 1;
}

static void skip_lines(FILE *f, int n)
{
  char buf[512];
  while (n-- > 0) {
    /* a line longer than the buffer is consumed in pieces, like fgets-based skipping */
    if (!fgets(buf, (int) sizeof buf, f)) return;
    while (!strchr(buf, '\n')) {
      if (!fgets(buf, (int) sizeof buf, f)) return;
    }
  }
}

int pdfs_vti_read(const char *path, pdfs_phi *pf)
{
  if (!path || !pf) return PDFS_ERR_INVALID;
  memset(pf, 0, sizeof(*pf));
  FILE *f = fopen(path, "r");
  if (!f) return PDFS_ERR_IO;
  char line[4096];
  double d[6];
  int found = 0;
  while (fgets(line, (int) sizeof line, f)) {
    if (strstr(line, "ImageData WholeExtent") && parse_header(line, d)) {
      found = 1;
      break;
    }
  }
  if (!found || !(d[0] >= 0 && d[1] >= 0 && d[2] >= 0) || d[0] > 1e7 || d[1] > 1e7 || d[2] > 1e7) {
    fclose(f);
    return PDFS_ERR_IO;
  }
  pf->x = (int) d[0] + 1;
  pf->y = (int) d[1] + 1;
  pf->z = (int) d[2] + 1;
  pf->dx = d[3];
  pf->dy = d[4];
  pf->dz = d[5];
  pf->F = 1.0;
  const long X = pf->x + 2, Y = pf->y + 2, Z = pf->z + 2;
  const size_t n = (size_t) X * (size_t) Y * (size_t) Z;
  pf->location = (int *) malloc(n * sizeof(int));
  pf->distance = (double *) malloc(n * sizeof(double));
  if (!pf->location || !pf->distance) {
    fclose(f);
    pdfs_phi_free(pf);
    return PDFS_ERR_OOM;
  }
  /* data: from the top of the file skip 6 lines, interior locations, skip the
   * rest of that line and one more, interior distances (vti_parser.c:112-125) */
  rewind(f);
  skip_lines(f, 6);
  int rc = PDFS_OK;
  for (long k = 0; k < Z && rc == PDFS_OK; k++)
    for (long j = 0; j < Y && rc == PDFS_OK; j++)
      for (long i = 0; i < X; i++) {
        int *t = pf->location + (k * Y + j) * X + i;
        if (i == 0 || i == X - 1 || j == 0 || j == Y - 1 || k == 0 || k == Z - 1) {
          *t = PDFS_BORDER_LOCATION;
        } else if (fscanf(f, "%d ", t) != 1) {
          rc = PDFS_ERR_IO;
          break;
        }
      }
  if (rc == PDFS_OK) skip_lines(f, 2);
  for (long k = 0; k < Z && rc == PDFS_OK; k++)
    for (long j = 0; j < Y && rc == PDFS_OK; j++)
      for (long i = 0; i < X; i++) {
        double *t = pf->distance + (k * Y + j) * X + i;
        if (i == 0 || i == X - 1 || j == 0 || j == Y - 1 || k == 0 || k == Z - 1) {
          *t = INFINITY;
        } else if (fscanf(f, "%lf ", t) != 1) {
          rc = PDFS_ERR_IO;
          break;
        }
      }
  fclose(f);
  if (rc != PDFS_OK) pdfs_phi_free(pf);
  return rc;
}

int pdfs_vti_write(const char *path, const pdfs_phi *pf)
{
  if (!path || !pf || !pf->distance || pf->x < 1 || pf->y < 1 || pf->z < 1) return PDFS_ERR_INVALID;
  FILE *fp = fopen(path, "w");
  if (!fp) return PDFS_ERR_IO;
  const int X = pf->x + 2, Y = pf->y + 2, Z = pf->z + 2;
  /* header and trailer of file_writer.c:156-189: extents of the halo-padded grid */
  fprintf(fp, "<?xml version=\"1.0\"?>\n");
  fprintf(fp, "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
  fprintf(fp, "\t<ImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"0 0 0\" Spacing=\" %f %f %f  \">\n", X - 1,
          Y - 1, Z - 1, pf->dx, pf->dy, pf->dz);
  fprintf(fp, "\t\t<Piece Extent=\"0 %d 0 %d 0 %d\">\n", X - 1, Y - 1, Z - 1);
  fprintf(fp, "\t\t\t<PointData Scalars=\"Distance Field\">\n");
  fprintf(fp, "\t\t\t\t<DataArray type=\"Float32\" Name=\"Distance Field\" format=\"ascii\">\n");
  const double *t = pf->distance;
  for (int k = 0; k < Z; k++) {
    for (int j = 0; j < Y; j++) {
      for (int i = 0; i < X; i++) fprintf(fp, "%f  ", *t++);
      fputc('\n', fp);
    }
    fputc('\n', fp);
  }
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  fprintf(fp, "\t\t\t</PointData>\n");
  fprintf(fp, "\t\t\t<CellData>\n");
  fprintf(fp, "\t\t\t</CellData>\n");
  fprintf(fp, "\t\t</Piece>\n");
  fprintf(fp, "\t</ImageData>\n");
  fprintf(fp, "</VTKFile>\n");
  return fclose(fp) == 0 ? PDFS_OK : PDFS_ERR_IO;
}

void pdfs_phi_free(pdfs_phi *pf)
{
  if (!pf) return;
  free(pf->location);
  free(pf->distance);
  pf->location = NULL;
  pf->distance = NULL;
}
