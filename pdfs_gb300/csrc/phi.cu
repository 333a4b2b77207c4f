// phi.cu -- the reference's distance-field pipeline on the GPU and the
// run_fsm drop-in (include/pdfs_phi.h).
//
// calc_dist_field (single_gpu_cuda/src/phi3D.c:107-126) runs three host passes
// around run_fsm; here they are device kernels on the uploaded arrays, so the
// field crosses the host boundary once in each direction.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/pdfs_phi.h"
#include "internal.h"

namespace pdfs {

// update_distance (phi3D.c:165-180): away from the border, a zero (or NaN)
// distance becomes the "unknown" value 90000.  The reference's extra clause
// (location 1 with an infinite distance -> -1) cannot trigger under its own
// guard (distance != inf), so it is left out.
__global__ void k_prepass(double *__restrict__ d, const int *__restrict__ l, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double v = d[i];
    if (l[i] != PDFS_BORDER_LOCATION && v != INFINITY) d[i] = (v > 0.0 || v < 0.0) ? v : PDFS_INTERIOR_DISTANCE;
  }
}

// set_distance_negative_inside (phi3D.c:190-205): inside nodes become -1.
__global__ void k_inside(double *__restrict__ d, const int *__restrict__ l, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (l[i] != PDFS_BORDER_LOCATION && d[i] != INFINITY && l[i] == 1) d[i] = -1.0;
}

// adjust_boundary (phi3D.c:221-242): every halo node takes the value of the
// nearest interior node (faces, edges and corners alike).  Sources are
// interior nodes, which the pass does not write, so the order is irrelevant.
__global__ void k_adjust_boundary(double *__restrict__ d, int X, int Y, int Z) {
  const int j = blockIdx.x, k = blockIdx.y;
  for (int i = threadIdx.x; i < X; i += blockDim.x) {
    const int I = i == X - 1 ? i - 1 : (i == 0 ? i + 1 : i);
    const int J = j == Y - 1 ? j - 1 : (j == 0 ? j + 1 : j);
    const int K = k == Z - 1 ? k - 1 : (k == 0 ? k + 1 : k);
    if (I != i || J != j || K != k)
      d[((size_t)k * Y + j) * X + i] = d[((size_t)K * Y + J) * X + I];
  }
}

}  // namespace pdfs

using namespace pdfs;

static int status_of(cudaError_t e) {
  if (e == cudaSuccess) return PDFS_OK;
  if (e == cudaErrorMemoryAllocation) return PDFS_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PDFS_ERR_NO_DEVICE;
  return PDFS_ERR_CUDA;
}

extern "C" int pdfs_calc_dist_field(pdfs_phi *pf, int rounds, const pdfs_opts *o_in, pdfs_stats *stats) {
  if (!pf || !pf->distance || !pf->location || rounds < 0) return PDFS_ERR_INVALID;
  pdfs_opts o;
  if (o_in)
    o = *o_in;
  else
    pdfs_default_opts(&o);
  if (rounds > 0) {
    o.fixed_sweeps = 8 * rounds;
    o.first_ordering = 1;
  }
  o.freeze = PDFS_FREEZE_NONE;  // the reference pipeline has no frozen mask
  const pdfs_grid g = {pf->x, pf->y, pf->z, pf->dx, pf->dy, pf->dz};
  pdfs_ctx *ctx = nullptr;
  int s = pdfs_ctx_create(&g, &o, &ctx);
  if (s) return s;
  const size_t n = (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2);
  double *dd = nullptr;
  int *dl = nullptr;
  cudaError_t e = cudaSuccess;
  const int grid = 2048, block = 256;
  pdfs_stats st;
  std::memset(&st, 0, sizeof(st));
  do {
    if ((e = cudaMalloc(&dd, n * 8)) != cudaSuccess) break;
    if ((e = cudaMalloc(&dl, n * 4)) != cudaSuccess) break;
    if ((e = cudaMemcpy(dd, pf->distance, n * 8, cudaMemcpyHostToDevice)) != cudaSuccess) break;
    if ((e = cudaMemcpy(dl, pf->location, n * 4, cudaMemcpyHostToDevice)) != cudaSuccess) break;
    k_prepass<<<grid, block>>>(dd, dl, n);
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) break;
    if ((s = pdfs_ctx_load(ctx, dd, nullptr)) != PDFS_OK) break;
    s = pdfs_ctx_run(ctx, &st);
    if (s != PDFS_OK && s != PDFS_ERR_NOT_CONVERGED) break;
    int s2 = pdfs_ctx_store(ctx, dd);
    if (s2) {
      s = s2;
      break;
    }
    k_inside<<<grid, block>>>(dd, dl, n);
    k_adjust_boundary<<<dim3(g.ny + 2, g.nz + 2), 128>>>(dd, g.nx + 2, g.ny + 2, g.nz + 2);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    if ((e = cudaMemcpy(pf->distance, dd, n * 8, cudaMemcpyDeviceToHost)) != cudaSuccess) break;
  } while (0);
  if (e != cudaSuccess) s = status_of(e);
  cudaFree(dd);
  cudaFree(dl);
  pdfs_ctx_destroy(ctx);
  st.status = s;
  if (stats) *stats = st;
  return s;
}

extern "C" void run_fsm(pdfs_phi *pf, int iterations) {
  if (!pf || !pf->distance || iterations < 1) {
    fprintf(stderr, "run_fsm: invalid argument\n");
    return;
  }
  const auto t0 = std::chrono::steady_clock::now();
  pdfs_opts o;
  pdfs_default_opts(&o);  // FP64, the reference's arithmetic, every node min-updated
  o.fixed_sweeps = 8 * iterations;
  o.first_ordering = 1;
  const pdfs_grid g = {pf->x, pf->y, pf->z, pf->dx, pf->dy, pf->dz};
  pdfs_stats st;
  const int s = pdfs_solve(&g, pf->distance, nullptr, &o, &st);
  if (s != PDFS_OK) {
    fprintf(stderr, "run_fsm: %s (%d); the field is unchanged\n", pdfs_status_string(s), s);
    return;
  }
  const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  printf("Parallel FSM time: %f s.\n", sec);  // the reference's report line (phi3D_fsm.cu:104)
  fflush(stdout);
}
