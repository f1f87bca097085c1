// dmath.cuh -- FP32 vector / quaternion helpers for the device path.
//
// Matrices are 3x4 row-major (12 floats, column 3 unused) like ODE's dMatrix3,
// so formulas carry over index-for-index from include/ode/odemath.h and
// ode/src/rotation.cpp. Expression order follows the reference; the compiler
// may contract products into FMAs (this path is FP32 and parity is checked
// against the FP64 oracle with a tolerance).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#define OG_HD __host__ __device__ __forceinline__
#define OG_D __device__ __forceinline__

namespace og {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kSqrt1_2 = 0.70710678118654752440f;

OG_HD float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
OG_HD float dot3s(const float* a, const float* b, int sa, int sb) {
  return a[0] * b[0] + a[sa] * b[sb] + a[2 * sa] * b[2 * sb];
}
OG_HD void cross3(float* r, const float* a, const float* b) {
  float r0 = a[1] * b[2] - a[2] * b[1];
  float r1 = a[2] * b[0] - a[0] * b[2];
  float r2 = a[0] * b[1] - a[1] * b[0];
  r[0] = r0; r[1] = r1; r[2] = r2;
}
// dMultiply0_331: res = A*b
OG_HD void mul0_331(float* res, const float* A, const float* b) {
  float r0 = dot3(A, b), r1 = dot3(A + 4, b), r2 = dot3(A + 8, b);
  res[0] = r0; res[1] = r1; res[2] = r2;
}
// dMultiply1_331: res = A^T*b
OG_HD void mul1_331(float* res, const float* A, const float* b) {
  float r0 = dot3s(A, b, 4, 1), r1 = dot3s(A + 1, b, 4, 1), r2 = dot3s(A + 2, b, 4, 1);
  res[0] = r0; res[1] = r1; res[2] = r2;
}
// dMultiply2_333: res = A*B^T
OG_HD void mul2_333(float* res, const float* A, const float* B) {
  mul0_331(res + 0, B, A + 0);
  mul0_331(res + 4, B, A + 4);
  mul0_331(res + 8, B, A + 8);
}
// dMultiply0_333: res = A*B
OG_HD void mul0_333(float* res, const float* A, const float* B) {
  mul1_331(res + 0, B, A + 0);
  mul1_331(res + 4, B, A + 4);
  mul1_331(res + 8, B, A + 8);
}

// _dSafeNormalize3 (ode/src/odemath.cpp:42-83)
OG_HD int safe_normalize3(float* a) {
  float aa0 = fabsf(a[0]), aa1 = fabsf(a[1]), aa2 = fabsf(a[2]);
  float m;
  if (aa1 > aa0) {
    m = (aa2 > aa1) ? aa2 : aa1;
  } else {
    if (aa2 > aa0) m = aa2;
    else {
      if (aa0 <= 0.f) { a[0] = 1.f; a[1] = 0.f; a[2] = 0.f; return 0; }
      m = aa0;
    }
  }
  a[0] /= m; a[1] /= m; a[2] /= m;
  float l = 1.0f / sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  a[0] *= l; a[1] *= l; a[2] *= l;
  return 1;
}
// _dSafeNormalize4 (ode/src/odemath.cpp:119-138)
OG_HD void normalize4(float* a) {
  float l = dot3(a, a) + a[3] * a[3];
  if (l > 0.f) {
    l = 1.0f / sqrtf(l);
    a[0] *= l; a[1] *= l; a[2] *= l; a[3] *= l;
  } else {
    a[0] = 1.f; a[1] = 0.f; a[2] = 0.f; a[3] = 0.f;
  }
}
// dPlaneSpace (ode/src/odemath.cpp:151-178)
OG_HD void plane_space(const float* n, float* p, float* q) {
  if (fabsf(n[2]) > kSqrt1_2) {
    float a = n[1] * n[1] + n[2] * n[2];
    float k = 1.0f / sqrtf(a);
    p[0] = 0.f; p[1] = -n[2] * k; p[2] = n[1] * k;
    q[0] = a * k; q[1] = -n[0] * p[2]; q[2] = n[0] * p[1];
  } else {
    float a = n[0] * n[0] + n[1] * n[1];
    float k = 1.0f / sqrtf(a);
    p[0] = -n[1] * k; p[1] = n[0] * k; p[2] = 0.f;
    q[0] = -n[2] * p[1]; q[1] = n[2] * p[0]; q[2] = a * k;
  }
}
// dRfromQ (ode/src/rotation.cpp:236-255)
OG_HD void r_from_q(float* R, const float* q) {
  float qq1 = 2.f * q[1] * q[1], qq2 = 2.f * q[2] * q[2], qq3 = 2.f * q[3] * q[3];
  R[0] = 1.f - qq2 - qq3; R[1] = 2.f * (q[1] * q[2] - q[0] * q[3]); R[2] = 2.f * (q[1] * q[3] + q[0] * q[2]); R[3] = 0.f;
  R[4] = 2.f * (q[1] * q[2] + q[0] * q[3]); R[5] = 1.f - qq1 - qq3; R[6] = 2.f * (q[2] * q[3] - q[0] * q[1]); R[7] = 0.f;
  R[8] = 2.f * (q[1] * q[3] - q[0] * q[2]); R[9] = 2.f * (q[2] * q[3] + q[0] * q[1]); R[10] = 1.f - qq1 - qq2; R[11] = 0.f;
}
// dQMultiply0/1/2/3 (ode/src/rotation.cpp:191-226)
OG_HD void qmul0(float* qa, const float* qb, const float* qc) {
  qa[0] = qb[0] * qc[0] - qb[1] * qc[1] - qb[2] * qc[2] - qb[3] * qc[3];
  qa[1] = qb[0] * qc[1] + qb[1] * qc[0] + qb[2] * qc[3] - qb[3] * qc[2];
  qa[2] = qb[0] * qc[2] + qb[2] * qc[0] + qb[3] * qc[1] - qb[1] * qc[3];
  qa[3] = qb[0] * qc[3] + qb[3] * qc[0] + qb[1] * qc[2] - qb[2] * qc[1];
}
OG_HD void qmul1(float* qa, const float* qb, const float* qc) {
  qa[0] = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
  qa[1] = qb[0] * qc[1] - qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
  qa[2] = qb[0] * qc[2] - qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
  qa[3] = qb[0] * qc[3] - qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
}
OG_HD void qmul2(float* qa, const float* qb, const float* qc) {
  qa[0] = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
  qa[1] = -qb[0] * qc[1] + qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
  qa[2] = -qb[0] * qc[2] + qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
  qa[3] = -qb[0] * qc[3] + qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
}
OG_HD void qmul3(float* qa, const float* qb, const float* qc) {
  qa[0] = qb[0] * qc[0] - qb[1] * qc[1] - qb[2] * qc[2] - qb[3] * qc[3];
  qa[1] = -qb[0] * qc[1] - qb[1] * qc[0] + qb[2] * qc[3] - qb[3] * qc[2];
  qa[2] = -qb[0] * qc[2] - qb[2] * qc[0] + qb[3] * qc[1] - qb[1] * qc[3];
  qa[3] = -qb[0] * qc[3] - qb[3] * qc[0] + qb[1] * qc[2] - qb[2] * qc[1];
}

// ---------------------------------------------------------------------------
// ODE's RNG (ode/src/misc.cpp:33-117): 32-bit LCG x -> 1664525 x + 1013904223,
// and dRandInt's xor-fold + modulus. lcg_jump advances by k calls in O(log k)
// by composing the affine map (a, c) with itself.
OG_HD unsigned lcg_next(unsigned s) { return 1664525u * s + 1013904223u; }
OG_HD unsigned lcg_jump(unsigned s, unsigned k) {
  unsigned a = 1664525u, c = 1013904223u;   // map x -> a x + c
  unsigned A = 1u, Cc = 0u;                 // accumulated map
  while (k) {
    if (k & 1u) { A = a * A; Cc = a * Cc + c; }
    c = a * c + c;
    a = a * a;
    k >>= 1;
  }
  return A * s + Cc;
}
OG_HD int rand_int_from(unsigned r, int n) {
  const unsigned un = (unsigned)n;
  if (un <= 0x10u) {
    r ^= (r >> 16); r ^= (r >> 8); r ^= (r >> 4);
    if (un <= 0x2u) { r ^= (r >> 2); r ^= (r >> 1); }
    else if (un <= 0x4u) { r ^= (r >> 2); }
  } else if (un <= 0x100u) {
    r ^= (r >> 16); r ^= (r >> 8);
  } else if (un <= 0x10000u) {
    r ^= (r >> 16);
  }
  return (int)(r % un);
}

}  // namespace og
