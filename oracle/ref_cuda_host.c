/* ref_cuda_host.c -- runs the reference's own CUDA sweep kernel on the GPU
 * (test infrastructure only: the plain-FP64 GPU comparator and a second
 * oracle for the GPU tests and the benchmark's reference legs).
 *
 * The kernel is fast_sweep_kernel of single_gpu_cuda/src/phi3D_fsm.cu:199-233
 * (with its solve_eikonal, :249-295), compiled unmodified from the reference's
 * sources into a cubin by `make -C oracle refcu`; nothing of it is copied
 * here.  This file is the host side: the reference's level loop
 * (phi3D_fsm.cu:127-190, one launch per hyperplane x+y+z = level, a device
 * synchronisation after each) and its pitched device copy of the field
 * (phi3D_fsm.cu:64-98), restated on the CUDA driver API so that the cubin
 * built from the reference's sources runs on any host architecture.
 *
 * Field: the reference layout, (nx+2)(ny+2)(nz+2) doubles, x fastest.
 */
#include <cuda.h>
#include <stddef.h>
#include <stdio.h>
#include <string.h>

/* The kernel's by-value parameters.  Their layouts are the CUDA runtime's
 * cudaPitchedPtr (driver_types.h) and the reference's SweepInfo
 * (single_gpu_cuda/src/phi3D_fsm.h:53-66): they must stay alike. */
typedef struct {
  void *ptr;
  size_t pitch, xsize, ysize;
} rc_pitched;
typedef struct {
  int level, xDim, yDim, zDim, xOffSet, yOffset, xSweepOff, ySweepOff, zSweepOff;
  double dx, dy, dz;
} rc_sweep;

/* The kernel's symbol: fast_sweep_kernel(cudaPitchedPtr, SweepInfo). */
static const char *kKernel = "_Z17fast_sweep_kernel14cudaPitchedPtr9SweepInfo";

static CUcontext g_ctx;
static CUmodule g_mod;
static CUfunction g_fn;
static char g_err[256];

static int fail(const char *what, CUresult r) {
  const char *s = NULL;
  cuGetErrorString(r, &s);
  snprintf(g_err, sizeof g_err, "%s: %s", what, s ? s : "?");
  return (int)r ? (int)r : -1;
}
#define RC(call)                         \
  do {                                   \
    CUresult r_ = (call);                \
    if (r_ != CUDA_SUCCESS) return fail(#call, r_); \
  } while (0)

const char *rc_error(void) { return g_err; }

/* Loads the cubin on device 0's primary context (the one the CUDA runtime
 * uses, so the comparator shares the device with the library under test). */
int rc_open(const char *cubin) {
  CUdevice dev;
  if (g_fn) {
    RC(cuModuleUnload(g_mod));
    g_fn = NULL;
  }
  RC(cuInit(0));
  RC(cuDeviceGet(&dev, 0));
  RC(cuDevicePrimaryCtxRetain(&g_ctx, dev));
  RC(cuCtxSetCurrent(g_ctx));
  RC(cuModuleLoad(&g_mod, cubin));
  RC(cuModuleGetFunction(&g_fn, g_mod, kKernel));
  return 0;
}

static int idiv_up(int a, int b) { return (a % b) ? a / b + 1 : a / b; }

/* Runs nsweeps orderings, the first being `first` (1..8), then first+1, ...
 * wrapping after 8 -- the reference's round is first = 1, nsweeps = 8
 * (phi3D_fsm.cu:148-189).  sync_each: synchronise after every level launch,
 * as the reference does (phi3D_fsm.cu:183); 0 queues the launches on one
 * stream instead.  ms_sweeps: device time of the sweeps alone (events);
 * ms_total: the whole call, allocation and copies included. */
int rc_run(double *dist, int nx, int ny, int nz, double dx, double dy, double dz, int first, int nsweeps,
           int sync_each, double *ms_sweeps, double *ms_total) {
  const int mesh = 3;
  const int X = nx + 2, Y = ny + 2, Z = nz + 2;
  CUdeviceptr d = 0;
  size_t pitch = 0;
  CUevent e0, e1, t0, t1;
  if (!g_fn) {
    snprintf(g_err, sizeof g_err, "rc_open was not called");
    return -1;
  }
  if (first < 1 || first > 8 || nsweeps < 0 || nx < 1 || ny < 1 || nz < 1) {
    snprintf(g_err, sizeof g_err, "bad arguments");
    return -1;
  }
  RC(cuCtxSetCurrent(g_ctx));
  RC(cuEventCreate(&t0, CU_EVENT_DEFAULT));
  RC(cuEventCreate(&t1, CU_EVENT_DEFAULT));
  RC(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  RC(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  RC(cuEventRecord(t0, 0));
  /* the pitched 3D allocation and copy of phi3D_fsm.cu:79-90 */
  RC(cuMemAllocPitch(&d, &pitch, (size_t)X * sizeof(double), (size_t)Y * Z, sizeof(double)));
  CUDA_MEMCPY2D cp;
  memset(&cp, 0, sizeof cp);
  cp.srcMemoryType = CU_MEMORYTYPE_HOST;
  cp.srcHost = dist;
  cp.srcPitch = (size_t)X * sizeof(double);
  cp.dstMemoryType = CU_MEMORYTYPE_DEVICE;
  cp.dstDevice = d;
  cp.dstPitch = pitch;
  cp.WidthInBytes = (size_t)X * sizeof(double);
  cp.Height = (size_t)Y * Z;
  RC(cuMemcpy2D(&cp));

  rc_pitched pp = {(void *)(size_t)d, pitch, (size_t)X * sizeof(double), (size_t)Y};
  rc_sweep sw;
  memset(&sw, 0, sizeof sw);
  sw.xDim = nx;
  sw.yDim = ny;
  sw.zDim = nz;
  sw.dx = dx;
  sw.dy = dy;
  sw.dz = dz;
  const int total = nx + ny + nz;
  RC(cuEventRecord(e0, 0));
  for (int s = 0; s < nsweeps; ++s) {
    const int sc = (first - 1 + s) % 8 + 1;
    /* the ordering table of phi3D_fsm.cu:149-159 */
    const int start = (sc == 2 || sc == 5 || sc == 7 || sc == 8) ? total : mesh;
    const int end = (start == mesh) ? total + 1 : mesh - 1;
    const int incr = start == mesh;
    sw.xSweepOff = (sc == 4 || sc == 8) ? nx + 1 : 0;
    sw.ySweepOff = (sc == 2 || sc == 6) ? ny + 1 : 0;
    sw.zSweepOff = (sc == 3 || sc == 7) ? nz + 1 : 0;
    for (int level = start; level != end; level = incr ? level + 1 : level - 1) {
      /* the level's x and y ranges and launch shape (phi3D_fsm.cu:161-176) */
      const int xs = level - (ny + nz) > 1 ? level - (ny + nz) : 1;
      const int ys = level - (nx + nz) > 1 ? level - (nx + nz) : 1;
      const int xe = nx < level - (mesh - 1) ? nx : level - (mesh - 1);
      const int ye = ny < level - (mesh - 1) ? ny : level - (mesh - 1);
      const int xr = xe - xs + 1, yr = ye - ys + 1;
      unsigned bx = 16, by = 16;
      if (xr * yr < 256) {
        bx = (unsigned)xr;
        by = (unsigned)yr;
      }
      sw.level = level;
      sw.xOffSet = xs;
      sw.yOffset = ys;
      void *args[2] = {&pp, &sw};
      RC(cuLaunchKernel(g_fn, (unsigned)idiv_up(xr, (int)bx), (unsigned)idiv_up(yr, (int)by), 1, bx, by, 1, 0, 0,
                        args, NULL));
      if (sync_each) RC(cuCtxSynchronize());
    }
  }
  RC(cuEventRecord(e1, 0));
  cp.srcMemoryType = CU_MEMORYTYPE_DEVICE;
  cp.srcDevice = d;
  cp.srcHost = NULL;
  cp.srcPitch = pitch;
  cp.dstMemoryType = CU_MEMORYTYPE_HOST;
  cp.dstHost = dist;
  cp.dstDevice = 0;
  cp.dstPitch = (size_t)X * sizeof(double);
  RC(cuMemcpy2D(&cp));
  RC(cuMemFree(d));
  RC(cuEventRecord(t1, 0));
  RC(cuEventSynchronize(t1));
  float ms = 0.f;
  RC(cuEventElapsedTime(&ms, e0, e1));
  if (ms_sweeps) *ms_sweeps = ms;
  RC(cuEventElapsedTime(&ms, t0, t1));
  if (ms_total) *ms_total = ms;
  cuEventDestroy(e0);
  cuEventDestroy(e1);
  cuEventDestroy(t0);
  cuEventDestroy(t1);
  return 0;
}
