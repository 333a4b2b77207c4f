/*
 * fsm_oracle.c -- CPU restatement of the parallel Fast Sweeping Method (FSM)
 * for |grad u| = 1, used ONLY as test infrastructure: the checker for the
 * GPU solver in tests, in the smoke check and as the CPU baseline leg of the
 * benchmark.  Nothing in the product links or calls this file.
 *
 * Parity is pinned: tests/golden/ holds fixtures produced by the reference's
 * own solver (mpi_openacc/src/phi3D_fsm.c compiled unmodified by
 * oracle/Makefile into oracle/_ref/), and the CPU test suite checks this
 * restatement against them bit for bit.
 *
 * Field layout (same as the reference, mpi_openacc/src/phi3D_fsm.c:86-112):
 * halo-padded (nx+2)*(ny+2)*(nz+2) doubles, x fastest, then y, then z;
 * interior nodes have 1-based coordinates 1..n on each axis.
 *
 * Arithmetic: the local solver evaluates exactly the expression trees of
 * solveEikonal (mpi_openacc/src/phi3D_fsm.c:132-182).  Compile with
 * -ffp-contract=off so that no multiply-add is fused (gcc on aarch64 fuses
 * by default).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MIN(a, b) ((a) < (b) ? (a) : (b))
#define ORC_MAX(a, b) ((a) > (b) ? (a) : (b))

/* Godunov upwind value from the three axis minima m[] with spacings d[].
 * Follows mpi_openacc/src/phi3D_fsm.c:142-179 (bubble sort with strict '>',
 * then 1-, 2- or 3-term solve in the reference's expanded form).  Returns the
 * candidate value only; the caller applies min(old, new) or min(cap, new). */
double orc_godunov(double mx, double my, double mz, double dx, double dy, double dz)
{
  double m[3] = {mx, my, mz};
  double d[3] = {dx, dy, dz};
  /* bubble sort: passes (0,1),(1,2) then (0,1) -- phi3D_fsm.c:148-159 */
  for (int i = 1; i < 3; i++) {
    for (int j = 0; j < 3 - i; j++) {
      if (m[j] > m[j + 1]) {
        double tm = m[j], td = d[j];
        m[j] = m[j + 1];
        d[j] = d[j + 1];
        m[j + 1] = tm;
        d[j + 1] = td;
      }
    }
  }
  double m2_0 = m[0] * m[0], m2_1 = m[1] * m[1], m2_2 = m[2] * m[2];
  double d2_0 = d[0] * d[0], d2_1 = d[1] * d[1], d2_2 = d[2] * d[2];

  double u = m[0] + d[0]; /* 1-term, phi3D_fsm.c:165 */
  if (u > m[1]) {         /* 2-term, phi3D_fsm.c:166-168 */
    double s = sqrt(-m2_0 + 2 * m[0] * m[1] - m2_1 + d2_0 + d2_1);
    u = (m[1] * d2_0 + m[0] * d2_1 + d[0] * d[1] * s) / (d2_0 + d2_1);
    if (u > m[2]) { /* 3-term, phi3D_fsm.c:170-177 */
      double a = sqrt(-m2_0 * d2_1 - m2_0 * d2_2 + 2 * m[0] * m[1] * d2_2 - m2_1 * d2_0
                      - m2_1 * d2_2 + 2 * m[0] * m[2] * d2_1 - m2_2 * d2_0 - m2_2 * d2_1
                      + 2 * m[1] * m[2] * d2_0 + d2_0 * d2_1 + d2_0 * d2_2 + d2_1 * d2_2);
      u = (m[2] * d2_0 * d2_1 + m[1] * d2_0 * d2_2 + m[0] * d2_1 * d2_2 + d[0] * d[1] * d[2] * a)
          / (d2_0 * d2_1 + d2_0 * d2_2 + d2_1 * d2_2);
    }
  }
  return u;
}

/* Sweep-direction table of makeSweepInfo (mpi_openacc/src/phi3D_fsm.c:195-221):
 * reflection offsets and level direction for ordering sn in 1..8. */
typedef struct {
  int xso, yso, zso; /* reflection offsets: index = |coord - off| */
  int descending;    /* levels run from nx+ny+nz down to 3 */
} orc_order;

static orc_order orc_make_order(int nx, int ny, int nz, int sn)
{
  orc_order o;
  o.xso = (sn == 4 || sn == 8) ? nx + 1 : 0;
  o.yso = (sn == 2 || sn == 6) ? ny + 1 : 0;
  o.zso = (sn == 3 || sn == 7) ? nz + 1 : 0;
  o.descending = (sn == 2 || sn == 5 || sn == 7 || sn == 8);
  return o;
}

/* mode 0: u = min(u, G)            (plain FSM, phi3D_fsm.c:181)
 * mode 1: u = min(cap, G)          (replace-update used by the FP64 polish)
 * frozen: optional byte mask in the field layout; nonzero = never updated.
 * Returns max |u_new - u_old| over the sweep (0 when nothing changed). */
static double orc_sweep_impl(int nx, int ny, int nz, double dx, double dy, double dz, double *u,
                             const uint8_t *frozen, const double *cap, int mode, int sn, int nthreads)
{
  const long extX = nx + 2;
  const long extXY = extX * (ny + 2);
  orc_order o = orc_make_order(nx, ny, nz, sn);
  const int first = 3, last = nx + ny + nz;
  double maxchg = 0.0;
  (void) nthreads;
  for (int step = 0; step <= last - first; step++) {
    /* hyperplane x+y+z = level, phi3D_fsm.c:92-117 */
    int level = o.descending ? last - step : first + step;
    int xs = ORC_MAX(1, level - (ny + nz));
    int ys = ORC_MAX(1, level - (nx + nz));
    int xe = ORC_MIN(nx, level - 2);
    int ye = ORC_MIN(ny, level - 2);
    double lvlmax = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(max : lvlmax) num_threads(nthreads) if (nthreads > 1 && (xe - xs) > 8)
#endif
    for (int x = xs; x <= xe; x++) {
      long k = labs((long) x - o.xso);
      for (int y = ys; y <= ye; y++) {
        int z = level - (x + y);
        if (z > 0 && z <= nz) {
          long j = labs((long) y - o.yso);
          long i = labs((long) z - o.zso);
          long idx = i * extXY + j * extX + k;
          if (frozen && frozen[idx]) continue;
          double old = u[idx];
          double mx = ORC_MIN(u[idx - 1], u[idx + 1]);
          double my = ORC_MIN(u[idx - extX], u[idx + extX]);
          double mz = ORC_MIN(u[idx - extXY], u[idx + extXY]);
          double g = orc_godunov(mx, my, mz, dx, dy, dz);
          double nv = mode == 0 ? ORC_MIN(old, g) : ORC_MIN(cap[idx], g);
          u[idx] = nv;
          double c = fabs(nv - old);
          if (c > lvlmax) lvlmax = c;
        }
      }
    }
    if (lvlmax > maxchg) maxchg = lvlmax;
  }
  return maxchg;
}

/* One ordering sn (1..8) of the plain FSM, as runFSM(pf, sn)
 * (mpi_openacc/src/phi3D_fsm.c:67,83-119); frozen may be NULL. */
double orc_sweep(int nx, int ny, int nz, double dx, double dy, double dz, double *u,
                 const uint8_t *frozen, int sn, int nthreads)
{
  return orc_sweep_impl(nx, ny, nz, dx, dy, dz, u, frozen, NULL, 0, sn, nthreads);
}

/* One ordering of the replace-update u = min(cap, G(neighbours)). */
double orc_sweep_replace(int nx, int ny, int nz, double dx, double dy, double dz, double *u,
                         const uint8_t *frozen, const double *cap, int sn, int nthreads)
{
  return orc_sweep_impl(nx, ny, nz, dx, dy, dz, u, frozen, cap, 1, sn, nthreads);
}

/* Plain FSM to convergence.  Orderings cycle 1..8; after every sweep the
 * sweep's max change is compared with tol and the solve stops at the first
 * sweep whose max change is <= tol (a sweep that changes nothing is a fixed
 * point of every ordering).  max_sweeps bounds the loop.  Returns the number
 * of sweeps run; *last_change receives the final sweep's max change. */
int orc_solve(int nx, int ny, int nz, double dx, double dy, double dz, double *u,
              const uint8_t *frozen, double tol, int max_sweeps, int nthreads, double *last_change)
{
  int s = 0;
  double c = 0.0;
  while (s < max_sweeps) {
    c = orc_sweep(nx, ny, nz, dx, dy, dz, u, frozen, (s % 8) + 1, nthreads);
    s++;
    if (c <= tol) break;
  }
  if (last_change) *last_change = c;
  return s;
}

/* ---------------------------------------------------------------------------
 * FP32 restatement of the shifted-form local solver used by the GPU FP32
 * sweeps: with sorted minima m0<=m1<=m2 and q_k = 1/h_k^2, a = m1-m0,
 * b = m2-m0 and v = u-m0:
 *   1 term: v = h0
 *   2 terms: v = (a q1 + sqrt(q0 + q1 - a^2 q0 q1)) / (q0 + q1)
 *   3 terms: v = (B + sqrt(max(0, B^2 - A C))) / A,
 *            A = q0+q1+q2, B = a q1 + b q2, C = a^2 q1 + b^2 q2 - 1.
 * The same quadratic as the reference's expanded form, rewritten in the
 * differences so that FP32 keeps its digits when m is large.
 * ------------------------------------------------------------------------- */
float orc_godunov_f32(float mx, float my, float mz, float hx, float hy, float hz)
{
  float m[3] = {mx, my, mz};
  float h[3] = {hx, hy, hz};
  for (int i = 1; i < 3; i++) {
    for (int j = 0; j < 3 - i; j++) {
      if (m[j] > m[j + 1]) {
        float tm = m[j], th = h[j];
        m[j] = m[j + 1];
        h[j] = h[j + 1];
        m[j + 1] = tm;
        h[j + 1] = th;
      }
    }
  }
  float u = m[0] + h[0];
  if (u > m[1]) {
    float q0 = 1.0f / (h[0] * h[0]), q1 = 1.0f / (h[1] * h[1]), q2 = 1.0f / (h[2] * h[2]);
    float a = m[1] - m[0];
    float disc = q0 + q1 - a * a * q0 * q1;
    if (disc < 0.0f) disc = 0.0f;
    u = m[0] + (a * q1 + sqrtf(disc)) / (q0 + q1);
    if (u > m[2]) {
      float b = m[2] - m[0];
      float A = q0 + q1 + q2, B = a * q1 + b * q2, C = a * a * q1 + b * b * q2 - 1.0f;
      float D = B * B - A * C;
      if (D < 0.0f) D = 0.0f;
      u = m[0] + (B + sqrtf(D)) / A;
    }
  }
  return u;
}

/* One FP32 ordering (min-update) on a float field in the same layout. */
float orc_sweep_f32(int nx, int ny, int nz, float dx, float dy, float dz, float *u,
                    const uint8_t *frozen, int sn)
{
  const long extX = nx + 2;
  const long extXY = extX * (ny + 2);
  orc_order o = orc_make_order(nx, ny, nz, sn);
  const int first = 3, last = nx + ny + nz;
  float maxchg = 0.0f;
  for (int step = 0; step <= last - first; step++) {
    int level = o.descending ? last - step : first + step;
    int xs = ORC_MAX(1, level - (ny + nz)), ys = ORC_MAX(1, level - (nx + nz));
    int xe = ORC_MIN(nx, level - 2), ye = ORC_MIN(ny, level - 2);
    for (int x = xs; x <= xe; x++) {
      long k = labs((long) x - o.xso);
      for (int y = ys; y <= ye; y++) {
        int z = level - (x + y);
        if (z > 0 && z <= nz) {
          long idx = labs((long) z - o.zso) * extXY + labs((long) y - o.yso) * extX + k;
          if (frozen && frozen[idx]) continue;
          float old = u[idx];
          float g = orc_godunov_f32(ORC_MIN(u[idx - 1], u[idx + 1]), ORC_MIN(u[idx - extX], u[idx + extX]),
                                    ORC_MIN(u[idx - extXY], u[idx + extXY]), dx, dy, dz);
          float nv = ORC_MIN(old, g);
          u[idx] = nv;
          if (old - nv > maxchg) maxchg = old - nv;
        }
      }
    }
  }
  return maxchg;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
