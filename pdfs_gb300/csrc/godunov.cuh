// godunov.cuh -- device local solvers of |grad u| = 1 (Godunov upwind update).
//
// Given the three axis minima m = (min(u[x-1],u[x+1]), min(u[y-1],u[y+1]),
// min(u[z-1],u[z+1])) and the spacings h, the update is the largest root u of
//     sum_k max(u - m_k, 0)^2 / h_k^2 = 1,
// found by sorting the minima and trying 1, 2 then 3 active terms
// (mpi_openacc/src/phi3D_fsm.c:132-182, single_gpu_cuda/src/phi3D_fsm.cu:249-295).
//
// Five variants:
//   god_ref64  -- the reference's own expanded expression trees, every
//                 operation an explicitly rounded intrinsic so nothing is fused:
//                 bit-identical to the reference's C compiled without contraction.
//   god_fast64 -- FP64, shifted form in the differences a = m1-m0, b = m2-m0.
//   god32s     -- FP32, same shifted form evaluated branch-free (the expanded
//                 form cancels catastrophically in FP32 once m is a few
//                 hundred cells).
//   god_mixed64 -- FP64 minima and result, FP32 increment (god32s on the
//                 FP64 differences to the smallest minimum).
//   god_pair    -- the same with FP32-pair (48-bit) minima and result.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace pdfs {

template <class T>
__device__ __forceinline__ void cswap(T &a, T &b) {
  T t = a;
  a = b;
  b = t;
}

// Per-sweep constants of the local solver.
struct GodConst64 {
  double h[3];   // spacings
  double h2[3];  // squared spacings
  double q[3];   // 1/h^2
  double qsum;   // q0+q1+q2
  double iqsum;  // 1/(q0+q1+q2)
};
struct GodConst32 {
  float h[3];
  float q[3];
  float iqsum;
  float iso_h, iso_2h2, iso_h2;  // isotropic shortcuts
};

// Reference arithmetic.  The bubble sort of solveEikonal (phi3D_fsm.c:148-159)
// is the compare-exchange sequence (0,1), (1,2), (0,1) with a strict '>', so
// ties keep axis order; the squared spacings travel with their minima (they
// are squared after the sort in the reference, which rounds identically).
__device__ __forceinline__ double god_ref64(double m0, double m1, double m2, const GodConst64 &k) {
  double d0 = k.h[0], d1 = k.h[1], d2 = k.h[2];
  double q0 = k.h2[0], q1 = k.h2[1], q2 = k.h2[2];
  if (m0 > m1) { cswap(m0, m1); cswap(d0, d1); cswap(q0, q1); }
  if (m1 > m2) { cswap(m1, m2); cswap(d1, d2); cswap(q1, q2); }
  if (m0 > m1) { cswap(m0, m1); cswap(d0, d1); cswap(q0, q1); }

  double u = __dadd_rn(m0, d0);  // phi3D_fsm.c:165
  if (u > m1) {
    const double m2_0 = __dmul_rn(m0, m0), m2_1 = __dmul_rn(m1, m1);
    // sqrt(-m2_0 + 2*m0*m1 - m2_1 + d2_0 + d2_1), left to right (phi3D_fsm.c:167)
    double t = __dadd_rn(-m2_0, __dmul_rn(__dmul_rn(2.0, m0), m1));
    t = __dsub_rn(t, m2_1);
    t = __dadd_rn(t, q0);
    t = __dadd_rn(t, q1);
    const double s = __dsqrt_rn(t);
    // (m1*d2_0 + m0*d2_1 + d0*d1*s) / (d2_0 + d2_1)  (phi3D_fsm.c:168)
    double num = __dadd_rn(__dadd_rn(__dmul_rn(m1, q0), __dmul_rn(m0, q1)), __dmul_rn(__dmul_rn(d0, d1), s));
    u = __ddiv_rn(num, __dadd_rn(q0, q1));
    if (u > m2) {
      const double m2_2 = __dmul_rn(m2, m2);
      // phi3D_fsm.c:171-173, a left-to-right chain of twelve terms
      double r = __dmul_rn(-m2_0, q1);
      r = __dsub_rn(r, __dmul_rn(m2_0, q2));
      r = __dadd_rn(r, __dmul_rn(__dmul_rn(__dmul_rn(2.0, m0), m1), q2));
      r = __dsub_rn(r, __dmul_rn(m2_1, q0));
      r = __dsub_rn(r, __dmul_rn(m2_1, q2));
      r = __dadd_rn(r, __dmul_rn(__dmul_rn(__dmul_rn(2.0, m0), m2), q1));
      r = __dsub_rn(r, __dmul_rn(m2_2, q0));
      r = __dsub_rn(r, __dmul_rn(m2_2, q1));
      r = __dadd_rn(r, __dmul_rn(__dmul_rn(__dmul_rn(2.0, m1), m2), q0));
      r = __dadd_rn(r, __dmul_rn(q0, q1));
      r = __dadd_rn(r, __dmul_rn(q0, q2));
      r = __dadd_rn(r, __dmul_rn(q1, q2));
      const double a = __dsqrt_rn(r);
      // phi3D_fsm.c:175-177
      double n3 = __dadd_rn(__dmul_rn(__dmul_rn(m2, q0), q1), __dmul_rn(__dmul_rn(m1, q0), q2));
      n3 = __dadd_rn(n3, __dmul_rn(__dmul_rn(m0, q1), q2));
      n3 = __dadd_rn(n3, __dmul_rn(__dmul_rn(__dmul_rn(d0, d1), d2), a));
      const double den = __dadd_rn(__dadd_rn(__dmul_rn(q0, q1), __dmul_rn(q0, q2)), __dmul_rn(q1, q2));
      u = __ddiv_rn(n3, den);
    }
  }
  return u;
}

// FP64 shifted form.  v = u - m0;  2 terms:
//   v = (a q1 + sqrt(q0 + q1 - a^2 q0 q1)) / (q0 + q1)
// 3 terms:  v = (B + sqrt(B^2 - A C)) / A  with A = q0+q1+q2,
//   B = a q1 + b q2,  C = a^2 q1 + b^2 q2 - 1.
__device__ __forceinline__ double god_fast64(double m0, double m1, double m2, const GodConst64 &k) {
  double h0 = k.h[0], h1 = k.h[1], h2 = k.h[2];
  double q0 = k.q[0], q1 = k.q[1], q2 = k.q[2];
  if (m0 > m1) { cswap(m0, m1); cswap(h0, h1); cswap(q0, q1); }
  if (m1 > m2) { cswap(m1, m2); cswap(h1, h2); cswap(q1, q2); }
  if (m0 > m1) { cswap(m0, m1); cswap(h0, h1); cswap(q0, q1); }
  double u = m0 + h0;
  if (u > m1) {
    const double a = m1 - m0;
    const double s = q0 + q1;
    const double disc = fma(-a * a, q0 * q1, s);
    u = m0 + (a * q1 + sqrt(fmax(disc, 0.0))) / s;
    if (u > m2) {
      const double b = m2 - m0;
      const double B = fma(a, q1, b * q2);
      const double Cc = fma(a * a, q1, fma(b * b, q2, -1.0));
      const double D = fma(B, B, -k.qsum * Cc);
      u = m0 + (B + sqrt(fmax(D, 0.0))) * k.iqsum;
    }
  }
  return u;
}

// FP32 shifted form evaluated branch-free: all three candidates are computed
// and the Godunov selection (1 term unless it exceeds the second minimum, 2
// terms unless they exceed the third) picks one.  Each candidate that can be
// selected is finite: u2 is only chosen when m1 < m0 + h (so a is finite), u3
// only when u2 > m2 (so b is finite); infinite minima only reach candidates
// that are not selected.
template <bool ISO>
__device__ __forceinline__ float god32s(float m0, float m1, float m2, const GodConst32 &k) {
  if (ISO) {
    const float lo = fminf(m0, m1), hi = fmaxf(m0, m1);
    const float mid = fminf(hi, m2);
    m2 = fmaxf(hi, m2);
    m0 = fminf(lo, mid);
    m1 = fmaxf(lo, mid);
    const float u1 = m0 + k.iso_h;
    const float a = m1 - m0;
    const float u2 = fmaf(0.5f, a + sqrtf(fmaxf(fmaf(-a, a, k.iso_2h2), 0.0f)), m0);
    const float b = m2 - m0;
    const float s = a + b;
    const float cc = fmaf(a, a, fmaf(b, b, -k.iso_h2));
    const float u3 = fmaf(s + sqrtf(fmaxf(fmaf(s, s, -3.0f * cc), 0.0f)), 1.0f / 3.0f, m0);
    return (u1 <= m1) ? u1 : ((u2 <= m2) ? u2 : u3);
  } else {
    float h0 = k.h[0], h1 = k.h[1], h2 = k.h[2];
    float q0 = k.q[0], q1 = k.q[1], q2 = k.q[2];
    if (m0 > m1) { cswap(m0, m1); cswap(h0, h1); cswap(q0, q1); }
    if (m1 > m2) { cswap(m1, m2); cswap(h1, h2); cswap(q1, q2); }
    if (m0 > m1) { cswap(m0, m1); cswap(h0, h1); cswap(q0, q1); }
    const float u1 = m0 + h0;
    const float a = m1 - m0;
    const float sq = q0 + q1;
    const float u2 = m0 + __fdividef(fmaf(a, q1, sqrtf(fmaxf(fmaf(-a * a, q0 * q1, sq), 0.0f))), sq);
    const float b = m2 - m0;
    const float B = fmaf(a, q1, b * q2);
    const float Cc = fmaf(a * a, q1, fmaf(b * b, q2, -1.0f));
    const float u3 = fmaf(B + sqrtf(fmaxf(fmaf(B, B, -(q0 + q1 + q2) * Cc), 0.0f)), k.iqsum, m0);
    return (u1 <= m1) ? u1 : ((u2 <= m2) ? u2 : u3);
  }
}

// FP64 field, FP32 increment.  The minima, the base (the smallest minimum)
// and the result stay FP64; only the increment above the base -- at most
// about h, so its FP32 rounding is about 1e-7 h -- is solved in FP32 from the
// FP64 differences.  Errors of a few 1e-8 h per update accumulate along a
// characteristic of n nodes to about 1e-7 of its length n h, so the fixed
// point lies within about 1e-7 relative of the FP64 one, at a handful of
// FP64 operations per update instead of a full FP64 quadratic (GB300 issues
// FP64 at 1/64 of the FP32 rate).
//
// GB300 runs every FP64 instruction -- add, compare, min/max and the
// double <-> float conversions alike -- at about 2 lane operations per clock
// per SM (measured), 1/64 of FP32.  So the mixed path does its compares on
// order-preserving integer keys and its conversions with integer bit
// arithmetic, and keeps exactly four FP64 additions per update: the two
// differences below, the final add, and the change in the sweep kernel.

// Integer key with the order of the doubles (-0 sorts below +0; no NaN here).
__device__ __forceinline__ long long dkey(double v) {
  const long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double kmin(double a, double b) { return dkey(a) < dkey(b) ? a : b; }

// x >= 0 (or +inf) to the nearest float (ties away from zero), by bit
// arithmetic; values below the float range flush to 0.
__device__ __forceinline__ float d2f_nonneg(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int de = (int)(hi >> 20);  // biased double exponent (sign bit is 0)
  const int fe = de - 1023 + 127;
  if (de == 0x7ff || fe >= 255) return __uint_as_float(0x7f800000u);
  if (fe <= 0) return 0.0f;
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  return __uint_as_float((((unsigned)fe << 23) | mant) + ((lo >> 28) & 1u));
}

// v >= 0 (a float) to the same value as a double, by bit arithmetic (exact;
// values below the normal float range flush to 0).
__device__ __forceinline__ double f2d_nonneg(float v) {
  const unsigned b = __float_as_uint(v);
  if (b < 0x00800000u) return 0.0;
  if (b >= 0x7f800000u) return __hiloint2double(0x7ff00000, 0);
  const unsigned de = (b >> 23) + (1023 - 127), m = b & 0x7fffffu;
  return __hiloint2double((int)((de << 20) | (m >> 3)), (int)(m << 29));
}

template <bool ISO>
__device__ __forceinline__ double god_mixed64(double m0, double m1, double m2, const GodConst32 &k) {
  const long long k0 = dkey(m0), k1 = dkey(m1), k2 = dkey(m2);
  const bool b0 = k0 <= k1 && k0 <= k2, b1 = !b0 && k1 <= k2;  // which axis holds the base
  const double base = b0 ? m0 : (b1 ? m1 : m2);
  if (((unsigned)__double2hiint(base) & 0x7ff00000u) == 0x7ff00000u) return base;  // no finite neighbour
  // the two other minima, in axis order; their differences to the base
  const double pa = b0 ? m1 : m0, pb = (b0 || b1) ? m2 : m1;
  const float ea = d2f_nonneg(pa - base), eb = d2f_nonneg(pb - base);
  const float e0 = b0 ? 0.0f : ea, e1 = b0 ? ea : (b1 ? 0.0f : eb), e2 = (b0 || b1) ? eb : 0.0f;
  return base + f2d_nonneg(god32s<ISO>(e0, e1, e2, k));
}

// ---- FP32 pairs ("double-float") --------------------------------------------------
// A value v is held as two floats hi + lo: hi is v rounded to float, |lo| <=
// ulp(hi) / 2, 48 significant bits in all.  A pair fills the 64 bits of an
// FP64 slot, hi in the low word and lo in the high word, so the FP64 layouts,
// tensor maps and kernels carry it unchanged.  The exact float sums are
// Knuth's TwoSum and Dekker's Fast2Sum (D. E. Knuth, TAOCP vol. 2, 4.2.2;
// T. J. Dekker, "A floating-point technique for extending the available
// precision", Numer. Math. 18, 1971); every operation is an explicitly
// rounded float intrinsic so none of them is contracted into an FMA.
__device__ __forceinline__ float p_hi(double v) { return __int_as_float(__double2loint(v)); }
__device__ __forceinline__ float p_lo(double v) { return __int_as_float(__double2hiint(v)); }
__device__ __forceinline__ double p_make(float hi, float lo) {
  return __hiloint2double(__float_as_int(lo), __float_as_int(hi));
}
// a < b for normalised pairs (hi = the value rounded to float)
__device__ __forceinline__ bool p_lt(double a, double b) {
  const float ah = p_hi(a), bh = p_hi(b);
  return ah < bh || (ah == bh && p_lo(a) < p_lo(b));
}
// the pair nearest a double (infinite, or beyond the float range: (hi, 0))
__device__ __forceinline__ double p_from_double(double d) {
  const float hi = (float)d;
  if (!(fabsf(hi) < INFINITY)) return p_make(hi, 0.0f);
  return p_make(hi, (float)(d - (double)hi));
}
// the reference's min(a, b) = a < b ? a : b, on pairs
__device__ __forceinline__ double pmin(double a, double b) { return p_lt(a, b) ? a : b; }
// a - b rounded to float (a, b not both infinite)
__device__ __forceinline__ float p_sub(double a, double b) {
  return __fadd_rn(__fsub_rn(p_hi(a), p_hi(b)), __fsub_rn(p_lo(a), p_lo(b)));
}
// b + x for a finite pair b and a float x >= 0: TwoSum of the high parts,
// the error folded into the low part, renormalised by Fast2Sum
__device__ __forceinline__ double p_add(double b, float x) {
  const float bh = p_hi(b), bl = p_lo(b);
  const float s = __fadd_rn(bh, x);
  const float bb = __fsub_rn(s, bh);
  const float e = __fadd_rn(__fsub_rn(bh, __fsub_rn(s, bb)), __fsub_rn(x, bb));
  const float t = __fadd_rn(bl, e);
  const float hi = __fadd_rn(s, t);
  return p_make(hi, __fsub_rn(t, __fsub_rn(hi, s)));
}

// FP32-pair field, FP32 increment: god_mixed64's scheme with the base, the
// minima and the result in pairs.  The differences to the base and the
// final sum run on the FP32 pipe, so no FP64 instruction is left.
//
// The three pairwise differences are formed first, all at once, and the
// base and the differences to it are chosen from their signs: for
// normalised pairs the sign of p_sub(a, b) is the sign of a - b (a tie gives
// 0, two infinite minima NaN, which counts as a tie), so the base and the
// increments are the ones an exact comparison would pick, with the choice
// no longer ahead of the subtractions on the update's dependency chain.
template <bool ISO>
__device__ __forceinline__ double god_pair(double m0, double m1, double m2, const GodConst32 &k) {
  const float d10 = p_sub(m1, m0), d20 = p_sub(m2, m0), d21 = p_sub(m2, m1);
  const bool b0 = !(d10 < 0.0f) && !(d20 < 0.0f);  // which axis holds the base
  const bool b1 = !b0 && !(d21 < 0.0f);
  const double base = b0 ? m0 : (b1 ? m1 : m2);
  // increments above the base, in axis order (the base's own is 0);
  // 0 - d is p_sub with the operands swapped, signed zeros included
  const float e0 = b0 ? 0.0f : (b1 ? __fsub_rn(0.0f, d10) : __fsub_rn(0.0f, d20));
  const float e1 = b0 ? d10 : (b1 ? 0.0f : __fsub_rn(0.0f, d21));
  const float e2 = b0 ? d20 : (b1 ? d21 : 0.0f);
  const double g = p_add(base, god32s<ISO>(e0, e1, e2, k));
  return p_hi(base) < INFINITY ? g : base;  // no finite neighbour: the base
}

}  // namespace pdfs
