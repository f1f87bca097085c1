/*
 * ode_oracle.c -- TEST INFRASTRUCTURE ONLY: the oracle. A CPU restatement of
 * ODE 0.12's primitive narrowphase + dWorldQuickStep step pipeline, written for
 * this project from the reference's behaviour (not copied), in FP64. Used by
 * tests/ as the checker, by __graft_entry__.smoke() to check one GPU step and
 * by bench.py's CPU-baseline leg. The product never links or calls it.
 *
 * Pinning: tests/test_oracle_vs_ref.py checks this file against the reference
 * ODE built from its own sources (oracle/Makefile -> oracle/_ref/) on seeded
 * scenes; results are required to be bit-identical in FP64 (the arithmetic
 * below follows the reference's operation order and is compiled without FMA
 * contraction). Golden vectors from the reference are committed under
 * tests/golden/ for hosts where the reference sources are absent.
 */
#define _GNU_SOURCE
#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include "ode_oracle.h"

typedef double real;
#define R_INF ((real)INFINITY)
#define R_PI 3.14159265358979323846
#define R_SQRT1_2 0.70710678118654752440

/* ------------------------------------------------------------------------ */
/* small vector helpers; each keeps the reference's evaluation order        */
/* (include/ode/odemath.h:44-225)                                          */

static inline real dot3(const real* a, const real* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline real dot3s(const real* a, const real* b, int sa, int sb) {
  return a[0] * b[0] + a[sa] * b[sb] + a[2 * sa] * b[2 * sb];
}
static inline void cross3(real* r, const real* a, const real* b) {
  real r0 = a[1] * b[2] - a[2] * b[1];
  real r1 = a[2] * b[0] - a[0] * b[2];
  real r2 = a[0] * b[1] - a[1] * b[0];
  r[0] = r0; r[1] = r1; r[2] = r2;
}
/* res = A*b, A is 3x4 row-major (dMultiply0_331) */
static inline void mul0_331(real* res, const real* A, const real* b) {
  real r0 = dot3(A, b), r1 = dot3(A + 4, b), r2 = dot3(A + 8, b);
  res[0] = r0; res[1] = r1; res[2] = r2;
}
/* res = A^T*b (dMultiply1_331) */
static inline void mul1_331(real* res, const real* A, const real* b) {
  real r0 = dot3s(A, b, 4, 1), r1 = dot3s(A + 1, b, 4, 1), r2 = dot3s(A + 2, b, 4, 1);
  res[0] = r0; res[1] = r1; res[2] = r2;
}
/* res = A*B^T (dMultiply2_333): row i of res is B * (row i of A) */
static inline void mul2_333(real* res, const real* A, const real* B) {
  mul0_331(res + 0, B, A + 0);
  mul0_331(res + 4, B, A + 4);
  mul0_331(res + 8, B, A + 8);
}
/* res = A*B (dMultiply0_333): row i of res is B^T * (row i of A) */
static inline void mul0_333(real* res, const real* A, const real* B) {
  mul1_331(res + 0, B, A + 0);
  mul1_331(res + 4, B, A + 4);
  mul1_331(res + 8, B, A + 8);
}

/* _dSafeNormalize3, ode/src/odemath.cpp:42-83 */
static int safe_normalize3(real* a) {
  real aa[3];
  int idx;
  aa[0] = fabs(a[0]); aa[1] = fabs(a[1]); aa[2] = fabs(a[2]);
  if (aa[1] > aa[0]) {
    idx = (aa[2] > aa[1]) ? 2 : 1;
  } else {
    if (aa[2] > aa[0]) idx = 2;
    else {
      if (aa[0] <= 0) { a[0] = 1; a[1] = 0; a[2] = 0; return 0; }
      idx = 0;
    }
  }
  a[0] /= aa[idx]; a[1] /= aa[idx]; a[2] /= aa[idx];
  real l = 1.0 / sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  a[0] *= l; a[1] *= l; a[2] *= l;
  return 1;
}
/* _dSafeNormalize4, ode/src/odemath.cpp:119-138 */
static void normalize4(real* a) {
  real l = dot3(a, a) + a[3] * a[3];
  if (l > 0) {
    l = 1.0 / sqrt(l);
    a[0] *= l; a[1] *= l; a[2] *= l; a[3] *= l;
  } else {
    a[0] = 1; a[1] = 0; a[2] = 0; a[3] = 0;
  }
}
/* dPlaneSpace, ode/src/odemath.cpp:151-178 */
static void plane_space(const real* n, real* p, real* q) {
  if (fabs(n[2]) > R_SQRT1_2) {
    real a = n[1] * n[1] + n[2] * n[2];
    real k = 1.0 / sqrt(a);
    p[0] = 0; p[1] = -n[2] * k; p[2] = n[1] * k;
    q[0] = a * k; q[1] = -n[0] * p[2]; q[2] = n[0] * p[1];
  } else {
    real a = n[0] * n[0] + n[1] * n[1];
    real k = 1.0 / sqrt(a);
    p[0] = -n[1] * k; p[1] = n[0] * k; p[2] = 0;
    q[0] = -n[2] * p[1]; q[1] = n[2] * p[0]; q[2] = a * k;
  }
}
/* dRfromQ, ode/src/rotation.cpp:236-255 */
static void r_from_q(real* R, const real* q) {
  real qq1 = 2 * q[1] * q[1], qq2 = 2 * q[2] * q[2], qq3 = 2 * q[3] * q[3];
  R[0] = 1 - qq2 - qq3; R[1] = 2 * (q[1] * q[2] - q[0] * q[3]); R[2] = 2 * (q[1] * q[3] + q[0] * q[2]); R[3] = 0;
  R[4] = 2 * (q[1] * q[2] + q[0] * q[3]); R[5] = 1 - qq1 - qq3; R[6] = 2 * (q[2] * q[3] - q[0] * q[1]); R[7] = 0;
  R[8] = 2 * (q[1] * q[3] - q[0] * q[2]); R[9] = 2 * (q[2] * q[3] + q[0] * q[1]); R[10] = 1 - qq1 - qq2; R[11] = 0;
}
/* dQMultiply0..3, ode/src/rotation.cpp:191-226 */
static void qmul0(real* qa, const real* qb, const real* qc) {
  qa[0] = qb[0] * qc[0] - qb[1] * qc[1] - qb[2] * qc[2] - qb[3] * qc[3];
  qa[1] = qb[0] * qc[1] + qb[1] * qc[0] + qb[2] * qc[3] - qb[3] * qc[2];
  qa[2] = qb[0] * qc[2] + qb[2] * qc[0] + qb[3] * qc[1] - qb[1] * qc[3];
  qa[3] = qb[0] * qc[3] + qb[3] * qc[0] + qb[1] * qc[2] - qb[2] * qc[1];
}
static void qmul1(real* qa, const real* qb, const real* qc) {
  qa[0] = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
  qa[1] = qb[0] * qc[1] - qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
  qa[2] = qb[0] * qc[2] - qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
  qa[3] = qb[0] * qc[3] - qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
}
static void qmul2(real* qa, const real* qb, const real* qc) {
  qa[0] = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
  qa[1] = -qb[0] * qc[1] + qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
  qa[2] = -qb[0] * qc[2] + qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
  qa[3] = -qb[0] * qc[3] + qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
}
static void qmul3(real* qa, const real* qb, const real* qc) {
  qa[0] = qb[0] * qc[0] - qb[1] * qc[1] - qb[2] * qc[2] - qb[3] * qc[3];
  qa[1] = -qb[0] * qc[1] - qb[1] * qc[0] + qb[2] * qc[3] - qb[3] * qc[2];
  qa[2] = -qb[0] * qc[2] - qb[2] * qc[0] + qb[3] * qc[1] - qb[1] * qc[3];
  qa[3] = -qb[0] * qc[3] - qb[3] * qc[0] + qb[1] * qc[2] - qb[2] * qc[1];
}
/* dRFrom2Axes, ode/src/rotation.cpp:94-133 (a zero-length input leaves R) */
static void r_from_2axes(real* R, real ax, real ay, real az, real bx, real by, real bz) {
  real l = sqrt(ax * ax + ay * ay + az * az);
  if (l <= 0) return;
  l = 1 / l;
  ax *= l; ay *= l; az *= l;
  real k = ax * bx + ay * by + az * bz;
  bx -= k * ax; by -= k * ay; bz -= k * az;
  l = sqrt(bx * bx + by * by + bz * bz);
  if (l <= 0) return;
  l = 1 / l;
  bx *= l; by *= l; bz *= l;
  R[0] = ax; R[4] = ay; R[8] = az;
  R[1] = bx; R[5] = by; R[9] = bz;
  R[2] = -by * az + ay * bz; R[6] = -bz * ax + az * bx; R[10] = -bx * ay + ax * by;
  R[3] = 0; R[7] = 0; R[11] = 0;
}
/* dQfromR, ode/src/rotation.cpp:258-306 */
static void q_from_r(real* q, const real* R) {
  real tr = R[0] + R[5] + R[10], s;
  if (tr >= 0) {
    s = sqrt(tr + 1);
    q[0] = 0.5 * s;
    s = 0.5 * (1 / s);
    q[1] = (R[9] - R[6]) * s; q[2] = (R[2] - R[8]) * s; q[3] = (R[4] - R[1]) * s;
    return;
  }
  int c;
  if (R[5] > R[0]) c = (R[10] > R[5]) ? 2 : 1;
  else c = (R[10] > R[0]) ? 2 : 0;
  if (c == 0) {
    s = sqrt((R[0] - (R[5] + R[10])) + 1);
    q[1] = 0.5 * s;
    s = 0.5 * (1 / s);
    q[2] = (R[1] + R[4]) * s; q[3] = (R[8] + R[2]) * s; q[0] = (R[9] - R[6]) * s;
  } else if (c == 1) {
    s = sqrt((R[5] - (R[10] + R[0])) + 1);
    q[2] = 0.5 * s;
    s = 0.5 * (1 / s);
    q[3] = (R[6] + R[9]) * s; q[1] = (R[1] + R[4]) * s; q[0] = (R[2] - R[8]) * s;
  } else {
    s = sqrt((R[10] - (R[0] + R[5])) + 1);
    q[3] = 0.5 * s;
    s = 0.5 * (1 / s);
    q[1] = (R[8] + R[2]) * s; q[2] = (R[6] + R[9]) * s; q[0] = (R[4] - R[1]) * s;
  }
}

/* ------------------------------------------------------------------------ */
/* RNG: ode/src/misc.cpp:31-117 (32-bit LCG, xor-folded modulus)            */

static _Thread_local unsigned int g_seed = 0;

static unsigned int rand_next(void) {
  g_seed = (unsigned int)(1664525u * g_seed + 1013904223u);
  return g_seed;
}
static int rand_int(int n) {
  const unsigned int un = (unsigned int)n;
  unsigned int r = rand_next();
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
void oracle_rand_set_seed(unsigned int s) { g_seed = s; }
unsigned int oracle_rand_get_seed(void) { return g_seed; }
int oracle_rand_int(int n) { return rand_int(n); }
int oracle_test_rand(void) {
  unsigned int old = g_seed;
  int ok = 1;
  g_seed = 0;
  if (rand_next() != 0x3c6ef35fu || rand_next() != 0x47502932u || rand_next() != 0xd1ccf6e9u ||
      rand_next() != 0xaaf95334u || rand_next() != 0x6252e503u)
    ok = 0;
  g_seed = old;
  return ok;
}

/* ------------------------------------------------------------------------ */
/* 3x3 SPD inverse by Cholesky, as dBodySetMass computes invI               */
/* (ode/src/ode.cpp:492-509 -> ode/src/matrix.cpp:121-230). A, Ainv: 3x4.   */

static int invert_pd3(const real* A, real* Ainv) {
  real L[12], recip[3];
  memcpy(L, A, sizeof(L));
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < i; ++j) {
      real sum = L[i * 4 + j];
      for (int k = 0; k < j; ++k) sum -= L[i * 4 + k] * L[j * 4 + k];
      L[i * 4 + j] = sum * recip[j];
    }
    real sum = L[i * 4 + i];
    for (int k = 0; k < i; ++k) sum -= L[i * 4 + k] * L[i * 4 + k];
    if (sum <= 0) return 0;
    real s = sqrt(sum);
    L[i * 4 + i] = s;
    recip[i] = 1.0 / s;
  }
  memset(Ainv, 0, 12 * sizeof(real));
  for (int c = 0; c < 3; ++c) {
    real x[3] = {0, 0, 0}, y[3];
    x[c] = 1;
    for (int r = 0; r < 3; ++r) {
      real sum = 0;
      for (int k = 0; k < r; ++k) sum += L[r * 4 + k] * y[k];
      y[r] = (x[r] - sum) / L[r * 4 + r];
    }
    for (int r = 2; r >= 0; --r) {
      real sum = 0;
      for (int k = r + 1; k < 3; ++k) sum += L[k * 4 + r] * x[k];
      x[r] = (y[r] - sum) / L[r * 4 + r];
    }
    for (int r = 0; r < 3; ++r) Ainv[r * 4 + c] = x[r];
  }
  return 1;
}

/* ------------------------------------------------------------------------ */
/* world model                                                              */

typedef struct {
  real pos[3], q[4], R[12];
  real lvel[3], avel[3], facc[3], tacc[3];
  real mass, invMass, I[12], invI[12];
  int flags;
  int tag;
  int* jl; int jl_n, jl_cap, jl_persist;   /* attached joints, attach order */
} OBody;

typedef struct {
  real vel, fmax, lostop, histop, fudge, normal_cfm, stop_erp, stop_cfm, bounce;
  int limit; real limit_err;
} OLimot;

typedef struct {
  int type;
  int b[2];          /* node[0].body, node[1].body after dJointAttach */
  int reverse;
  int tag;
  /* ball / hinge / hinge2 */
  real anchor1[4], anchor2[4], axis1[4], axis2[4], qrel[4];
  real erp, cfm;
  OLimot lm1, lm2;
  real c0, s0, v1[4], v2[4], susp_erp, susp_cfm;
  real offset[4];    /* slider, fixed */
  real qrel2[4];     /* universal (qrel holds qrel1) */
  /* angular motor: lm1 / lm2 / lm3 drive axes 0 / 1 / 2 */
  OLimot lm3;
  int am_num, am_mode, am_rel[3];
  real am_axis[3][4], am_ref1[4], am_ref2[4], am_angle[3];
  /* contact */
  odegpuSurface surf;
  real cpos[3], cnormal[3], cdepth;
  int the_m;
  real fb[12];       /* joint feedback f1 t1 f2 t2 */
} OJoint;

typedef struct {
  int type, body;
  real p[4];     /* sphere r / box sides / capsule r,len / plane */
  int surface;
  const odegpuHeightfield* hf;
  real hpos[3], hR[12];
} OGeom;

typedef struct {
  const odegpuScene* sc;
  int w, nb, ng, nj_persist;
  OBody* body;
  OGeom* geom;
  OJoint* joint; int nj, cap_j;
  real gravity[3], erp, cfm, sor_w, max_vel, min_depth, dt;
  int iterations, max_contacts;
  oracleTap* tap;
  int last_rows, last_islands;   /* rows and islands with rows of the last step */
} OWorld;

static void body_attach(OBody* b, int j) {
  if (b->jl_n == b->jl_cap) {
    b->jl_cap = b->jl_cap ? 2 * b->jl_cap : 8;
    b->jl = (int*)realloc(b->jl, b->jl_cap * sizeof(int));
  }
  b->jl[b->jl_n++] = j;
}

/* dJointAttach, ode/src/ode.cpp:1348-1399: a missing body1 moves to body2's
 * slot and sets the reverse flag; the joint is prepended on each body's list. */
static void joint_attach(OWorld* W, int j, int b1, int b2) {
  OJoint* J = &W->joint[j];
  if (b1 < 0) { b1 = b2; b2 = -1; J->reverse = 1; } else J->reverse = 0;
  J->b[0] = b1; J->b[1] = b2;
  if (b1 >= 0) body_attach(&W->body[b1], j);
  if (b2 >= 0) body_attach(&W->body[b2], j);
}

/* setAnchors / setAxes, ode/src/joints/joint.cpp:260-322 */
static void set_anchors(OWorld* W, OJoint* J, real x, real y, real z, real* a1, real* a2) {
  if (J->b[0] >= 0) {
    OBody* B1 = &W->body[J->b[0]];
    real q[4] = {x - B1->pos[0], y - B1->pos[1], z - B1->pos[2], 0};
    mul1_331(a1, B1->R, q);
    if (J->b[1] >= 0) {
      OBody* B2 = &W->body[J->b[1]];
      real q2[4] = {x - B2->pos[0], y - B2->pos[1], z - B2->pos[2], 0};
      mul1_331(a2, B2->R, q2);
    } else {
      a2[0] = x; a2[1] = y; a2[2] = z;
    }
  }
  a1[3] = 0; a2[3] = 0;
}
static void set_axes(OWorld* W, OJoint* J, real x, real y, real z, real* ax1, real* ax2) {
  if (J->b[0] >= 0) {
    real q[4] = {x, y, z, 0};
    safe_normalize3(q);
    if (ax1) { mul1_331(ax1, W->body[J->b[0]].R, q); ax1[3] = 0; }
    if (ax2) {
      if (J->b[1] >= 0) mul1_331(ax2, W->body[J->b[1]].R, q);
      else { ax2[0] = x; ax2[1] = y; ax2[2] = z; }
      ax2[3] = 0;
    }
  }
}
/* dxJointHinge::computeInitialRelativeRotation, ode/src/joints/hinge.cpp:378-396 */
static void hinge_qrel(OWorld* W, OJoint* J) {
  if (J->b[0] >= 0) {
    const real* q1 = W->body[J->b[0]].q;
    if (J->b[1] >= 0) qmul1(J->qrel, q1, W->body[J->b[1]].q);
    else { J->qrel[0] = q1[0]; J->qrel[1] = -q1[1]; J->qrel[2] = -q1[2]; J->qrel[3] = -q1[3]; }
  }
}
/* dxJointSlider::computeOffset, ode/src/joints/slider.cpp:380-398 */
static void slider_offset(OWorld* W, OJoint* J) {
  if (J->b[1] >= 0) {
    real c[3];
    for (int i = 0; i < 3; ++i) c[i] = W->body[J->b[0]].pos[i] - W->body[J->b[1]].pos[i];
    mul1_331(J->offset, W->body[J->b[1]].R, c);
  } else if (J->b[0] >= 0) {
    for (int i = 0; i < 3; ++i) J->offset[i] = W->body[J->b[0]].pos[i];
  }
}
/* dJointSetFixed, ode/src/joints/fixed.cpp:110-132 */
static void fixed_set(OWorld* W, OJoint* J) {
  if (J->b[0] >= 0) {
    if (J->b[1] >= 0) {
      real ofs[3];
      for (int i = 0; i < 3; ++i) ofs[i] = W->body[J->b[0]].pos[i] - W->body[J->b[1]].pos[i];
      mul1_331(J->offset, W->body[J->b[0]].R, ofs);
    } else {
      for (int i = 0; i < 3; ++i) J->offset[i] = W->body[J->b[0]].pos[i];
    }
  }
  hinge_qrel(W, J);   /* the fixed joint's computeInitialRelativeRotation is the same */
}
/* dxJointUniversal::getAxes, ode/src/joints/universal.cpp:55-70 */
static void universal_axes(OWorld* W, OJoint* J, real* ax1, real* ax2) {
  mul0_331(ax1, W->body[J->b[0]].R, J->axis1);
  if (J->b[1] >= 0) mul0_331(ax2, W->body[J->b[1]].R, J->axis2);
  else { ax2[0] = J->axis2[0]; ax2[1] = J->axis2[1]; ax2[2] = J->axis2[2]; }
}
/* dxJointUniversal::computeInitialRelativeRotations, ode/src/joints/universal.cpp:365-393 */
static void universal_qrels(OWorld* W, OJoint* J) {
  if (J->b[0] < 0) return;
  real ax1[3], ax2[3], qcross[4];
  real R[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  universal_axes(W, J, ax1, ax2);
  r_from_2axes(R, ax1[0], ax1[1], ax1[2], ax2[0], ax2[1], ax2[2]);
  q_from_r(qcross, R);
  qmul1(J->qrel, W->body[J->b[0]].q, qcross);
  r_from_2axes(R, ax2[0], ax2[1], ax2[2], ax1[0], ax1[1], ax1[2]);
  q_from_r(qcross, R);
  if (J->b[1] >= 0) qmul1(J->qrel2, W->body[J->b[1]].q, qcross);
  else for (int i = 0; i < 4; ++i) J->qrel2[i] = qcross[i];
}
/* dxJointAMotor::setEulerReferenceVectors, ode/src/joints/amotor.cpp:148-181
 * (without a second body reference2 is added to on every call) */
static void amotor_euler_refs(OWorld* W, OJoint* J) {
  if (J->b[0] < 0) return;
  const real* R1 = W->body[J->b[0]].R;
  if (J->b[1] >= 0) {
    const real* R2 = W->body[J->b[1]].R;
    real r[4];
    mul0_331(r, R2, J->am_axis[2]);
    mul1_331(J->am_ref1, R1, r);
    mul0_331(r, R1, J->am_axis[0]);
    mul1_331(J->am_ref2, R2, r);
  } else {
    real r[4] = {J->am_axis[2][0], J->am_axis[2][1], J->am_axis[2][2], J->am_axis[2][3]};
    mul1_331(J->am_ref1, R1, r);
    mul0_331(r, R1, J->am_axis[0]);
    for (int k = 0; k < 4; ++k) J->am_ref2[k] += r[k];
  }
}
/* dJointSetAMotorMode / NumAxes / Axis, ode/src/joints/amotor.cpp:260-323, :350-363 */
static void amotor_set_mode(OWorld* W, OJoint* J, int mode) {
  J->am_mode = mode;
  if (mode == 1) { J->am_num = 3; amotor_euler_refs(W, J); }
}
static void amotor_set_num(OJoint* J, int num) {
  if (J->am_mode == 1) J->am_num = 3;
  else J->am_num = num < 0 ? 0 : (num > 3 ? 3 : num);
}
static void amotor_set_axis(OWorld* W, OJoint* J, int anum, int rel, real x, real y, real z) {
  if (anum < 0) anum = 0;
  if (anum > 2) anum = 2;
  if (J->b[1] < 0 && rel == 2) rel = 1;
  J->am_rel[anum] = rel;
  real r[4] = {x, y, z, 0};
  real* a = J->am_axis[anum];
  if (rel > 0) {
    if (rel == 1) mul1_331(a, W->body[J->b[0]].R, r);
    else if (J->b[1] >= 0) mul1_331(a, W->body[J->b[1]].R, r);
    else for (int k = 0; k < 4; ++k) a[k] = r[k];
  } else {
    a[0] = r[0]; a[1] = r[1]; a[2] = r[2];
  }
  safe_normalize3(a);
  if (J->am_mode == 1) amotor_euler_refs(W, J);
}
/* dxJointAMotor::computeGlobalAxes, ode/src/joints/amotor.cpp:52-94 */
static void amotor_axes(OWorld* W, OJoint* J, real ax[3][4]) {
  const real* R1 = W->body[J->b[0]].R;
  if (J->am_mode == 1) {
    mul0_331(ax[0], R1, J->am_axis[0]);
    if (J->b[1] >= 0) mul0_331(ax[2], W->body[J->b[1]].R, J->am_axis[2]);
    else { ax[2][0] = J->am_axis[2][0]; ax[2][1] = J->am_axis[2][1]; ax[2][2] = J->am_axis[2][2]; }
    cross3(ax[1], ax[2], ax[0]);
    safe_normalize3(ax[1]);
    return;
  }
  for (int i = 0; i < J->am_num; ++i) {
    if (J->am_rel[i] == 1) mul0_331(ax[i], R1, J->am_axis[i]);
    else if (J->am_rel[i] == 2) {
      if (J->b[1] >= 0) mul0_331(ax[i], W->body[J->b[1]].R, J->am_axis[i]);
    } else {
      ax[i][0] = J->am_axis[i][0]; ax[i][1] = J->am_axis[i][1]; ax[i][2] = J->am_axis[i][2];
    }
  }
}
/* dxJointAMotor::computeEulerAngles, ode/src/joints/amotor.cpp:98-139 */
static void amotor_euler_angles(OWorld* W, OJoint* J, real ax[3][4]) {
  real ref1[3], ref2[3], q[3];
  mul0_331(ref1, W->body[J->b[0]].R, J->am_ref1);
  if (J->b[1] >= 0) mul0_331(ref2, W->body[J->b[1]].R, J->am_ref2);
  else { ref2[0] = J->am_ref2[0]; ref2[1] = J->am_ref2[1]; ref2[2] = J->am_ref2[2]; }
  cross3(q, ax[0], ref1);
  J->am_angle[0] = -atan2(dot3(ax[2], q), dot3(ax[2], ref1));
  cross3(q, ax[0], ax[1]);
  J->am_angle[1] = -atan2(dot3(ax[2], ax[0]), dot3(ax[2], q));
  cross3(q, ax[1], ax[2]);
  J->am_angle[2] = -atan2(dot3(ref2, ax[1]), dot3(ref2, q));
}
/* dxJointHinge2::getAxisInfo / makeV1andV2, ode/src/joints/hinge2.cpp:97-106, :184-210 */
static void hinge2_axis_info(OWorld* W, OJoint* J, real* ax1, real* ax2, real* axc, real* s, real* c) {
  mul0_331(ax1, W->body[J->b[0]].R, J->axis1);
  mul0_331(ax2, W->body[J->b[1]].R, J->axis2);
  cross3(axc, ax1, ax2);
  *s = sqrt(axc[0] * axc[0] + axc[1] * axc[1] + axc[2] * axc[2]);
  *c = dot3(ax1, ax2);
}
static void hinge2_make_v(OWorld* W, OJoint* J) {
  if (J->b[0] < 0) return;
  real ax1[4], ax2[4], v[4];
  mul0_331(ax1, W->body[J->b[0]].R, J->axis1);
  mul0_331(ax2, W->body[J->b[1]].R, J->axis2);
  if ((ax1[0] == 0 && ax1[1] == 0 && ax1[2] == 0) || (ax2[0] == 0 && ax2[1] == 0 && ax2[2] == 0) ||
      (ax1[0] == ax2[0] && ax1[1] == ax2[1] && ax1[2] == ax2[2]))
    return;
  real k = dot3(ax1, ax2);
  for (int i = 0; i < 3; ++i) ax2[i] -= k * ax1[i];
  safe_normalize3(ax2);
  cross3(v, ax1, ax2);
  mul1_331(J->v1, W->body[J->b[0]].R, ax2);
  mul1_331(J->v2, W->body[J->b[0]].R, v);
}
static void get_anchor(OWorld* W, OJoint* J, real* res, const real* a1) {
  if (J->b[0] >= 0) {
    OBody* B = &W->body[J->b[0]];
    mul0_331(res, B->R, a1);
    res[0] += B->pos[0]; res[1] += B->pos[1]; res[2] += B->pos[2];
  }
}
static void get_anchor2(OWorld* W, OJoint* J, real* res, const real* a2) {
  if (J->b[1] >= 0) {
    OBody* B = &W->body[J->b[1]];
    mul0_331(res, B->R, a2);
    res[0] += B->pos[0]; res[1] += B->pos[1]; res[2] += B->pos[2];
  } else {
    res[0] = a2[0]; res[1] = a2[1]; res[2] = a2[2];
  }
}

/* dxJointLimitMotor::init, ode/src/joints/joint.cpp:456-469 */
static void limot_init(OLimot* L, const OWorld* W) {
  L->vel = 0; L->fmax = 0; L->lostop = -R_INF; L->histop = R_INF; L->fudge = 1;
  L->normal_cfm = W->cfm; L->stop_erp = W->erp; L->stop_cfm = W->cfm; L->bounce = 0;
  L->limit = 0; L->limit_err = 0;
}
/* dxJointLimitMotor::set, ode/src/joints/joint.cpp:472-508, applied in the
 * order the harness applies the parameters. */
static void limot_set_all(OLimot* L, const double* p) {
  L->lostop = p[0];
  L->histop = p[1];
  L->vel = p[2];
  if (p[3] >= 0) L->fmax = p[3];
  if (p[4] >= 0 && p[4] <= 1) L->fudge = p[4];
  L->bounce = p[5];
  L->normal_cfm = p[6];
  L->stop_erp = p[7];
  L->stop_cfm = p[8];
}

/* ------------------------------------------------------------------------ */
/* colliders                                                                */

typedef struct { real pos[3], normal[3], depth; } OContact;

typedef struct {
  int type;
  const real* pos;   /* final_posr pos */
  const real* R;     /* final_posr R (3x4) */
  const real* p;     /* class parameters */
  const OGeom* g;
} GeomRef;

/* dCollideSpheres, ode/src/collision_util.cpp:38-67 */
static int collide_spheres(const real* p1, real r1, const real* p2, real r2, OContact* c) {
  real t[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
  real d = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
  if (d > (r1 + r2)) return 0;
  if (d <= 0) {
    c->pos[0] = p1[0]; c->pos[1] = p1[1]; c->pos[2] = p1[2];
    c->normal[0] = 1; c->normal[1] = 0; c->normal[2] = 0;
    c->depth = r1 + r2;
  } else {
    real d1 = 1.0 / d;
    c->normal[0] = (p1[0] - p2[0]) * d1;
    c->normal[1] = (p1[1] - p2[1]) * d1;
    c->normal[2] = (p1[2] - p2[2]) * d1;
    real k = 0.5 * (r2 - r1 - d);
    c->pos[0] = p1[0] + c->normal[0] * k;
    c->pos[1] = p1[1] + c->normal[1] * k;
    c->pos[2] = p1[2] + c->normal[2] * k;
    c->depth = r1 + r2 - d;
  }
  return 1;
}

/* dCollideSphereBox, ode/src/sphere.cpp:131-219 */
static int collide_sphere_box(const GeomRef* s, const GeomRef* b, OContact* c) {
  real l[3], t[4], p[3], q[3], r[3];
  int onborder = 0;
  const real* R = b->R;
  p[0] = s->pos[0] - b->pos[0];
  p[1] = s->pos[1] - b->pos[1];
  p[2] = s->pos[2] - b->pos[2];
  l[0] = b->p[0] * 0.5;
  t[0] = dot3s(p, R, 1, 4);
  if (t[0] < -l[0]) { t[0] = -l[0]; onborder = 1; }
  if (t[0] > l[0]) { t[0] = l[0]; onborder = 1; }
  l[1] = b->p[1] * 0.5;
  t[1] = dot3s(p, R + 1, 1, 4);
  if (t[1] < -l[1]) { t[1] = -l[1]; onborder = 1; }
  if (t[1] > l[1]) { t[1] = l[1]; onborder = 1; }
  t[2] = dot3s(p, R + 2, 1, 4);
  l[2] = b->p[2] * 0.5;
  if (t[2] < -l[2]) { t[2] = -l[2]; onborder = 1; }
  if (t[2] > l[2]) { t[2] = l[2]; onborder = 1; }
  if (!onborder) {
    real min_distance = l[0] - fabs(t[0]);
    int mini = 0;
    for (int i = 1; i < 3; i++) {
      real fd = l[i] - fabs(t[i]);
      if (fd < min_distance) { min_distance = fd; mini = i; }
    }
    c->pos[0] = s->pos[0]; c->pos[1] = s->pos[1]; c->pos[2] = s->pos[2];
    real tmp[3] = {0, 0, 0};
    tmp[mini] = (t[mini] > 0) ? 1.0 : -1.0;
    mul0_331(c->normal, R, tmp);
    c->depth = min_distance + s->p[0];
    return 1;
  }
  t[3] = 0;
  mul0_331(q, R, t);
  r[0] = p[0] - q[0]; r[1] = p[1] - q[1]; r[2] = p[2] - q[2];
  real depth = s->p[0] - sqrt(dot3(r, r));
  if (depth < 0) return 0;
  c->pos[0] = q[0] + b->pos[0];
  c->pos[1] = q[1] + b->pos[1];
  c->pos[2] = q[2] + b->pos[2];
  c->normal[0] = r[0]; c->normal[1] = r[1]; c->normal[2] = r[2];
  safe_normalize3(c->normal);
  c->depth = depth;
  return 1;
}

/* dCollideSpherePlane, ode/src/sphere.cpp:222-251 */
static int collide_sphere_plane(const GeomRef* s, const GeomRef* pl, OContact* c) {
  const real* P = pl->p;
  real k = dot3(s->pos, P);
  real depth = P[3] - k + s->p[0];
  if (depth >= 0) {
    c->normal[0] = P[0]; c->normal[1] = P[1]; c->normal[2] = P[2];
    c->pos[0] = s->pos[0] - P[0] * s->p[0];
    c->pos[1] = s->pos[1] - P[1] * s->p[0];
    c->pos[2] = s->pos[2] - P[2] * s->p[0];
    c->depth = depth;
    return 1;
  }
  return 0;
}

/* dLineClosestApproach, ode/src/collision_util.cpp:70-92 */
static void line_closest_approach(const real* pa, const real* ua, const real* pb, const real* ub,
                                  real* alpha, real* beta) {
  real p[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
  real uaub = dot3(ua, ub);
  real q1 = dot3(ua, p);
  real q2 = -dot3(ub, p);
  real d = 1 - uaub * uaub;
  if (d <= 0.0001) { *alpha = 0; *beta = 0; }
  else {
    d = 1.0 / d;
    *alpha = (q1 + uaub * q2) * d;
    *beta = (uaub * q1 + q2) * d;
  }
}

/* intersectRectQuad, ode/src/box.cpp:187-245: clip quad p against the
 * rectangle |x|<h[0], |y|<h[1] with the same point-emission order. */
static int intersect_rect_quad(const real h[2], real p[8], real ret[16]) {
  int nq = 4, nr = 0;
  real buffer[16];
  real* q = p;
  real* r = ret;
  for (int dir = 0; dir <= 1; dir++) {
    for (int sign = -1; sign <= 1; sign += 2) {
      real* pq = q;
      real* pr = r;
      nr = 0;
      for (int i = nq; i > 0; i--) {
        if (sign * pq[dir] < h[dir]) {
          pr[0] = pq[0]; pr[1] = pq[1];
          pr += 2; nr++;
          if (nr & 8) { q = r; goto done; }
        }
        real* nextq = (i > 1) ? pq + 2 : q;
        if ((sign * pq[dir] < h[dir]) ^ (sign * nextq[dir] < h[dir])) {
          pr[1 - dir] = pq[1 - dir] + (nextq[1 - dir] - pq[1 - dir]) / (nextq[dir] - pq[dir]) *
                                          (sign * h[dir] - pq[dir]);
          pr[dir] = sign * h[dir];
          pr += 2; nr++;
          if (nr & 8) { q = r; goto done; }
        }
        pq += 2;
      }
      q = r;
      r = (q == ret) ? buffer : ret;
      nq = nr;
    }
  }
done:
  if (q != ret) memcpy(ret, q, nr * 2 * sizeof(real));
  return nr;
}

/* cullPoints, ode/src/box.cpp:249-322 */
static void cull_points(int n, const real p[], int m, int i0, int iret[]) {
  int i, j;
  real a, cx, cy, q;
  if (n == 1) { cx = p[0]; cy = p[1]; }
  else if (n == 2) { cx = 0.5 * (p[0] + p[2]); cy = 0.5 * (p[1] + p[3]); }
  else {
    a = 0; cx = 0; cy = 0;
    for (i = 0; i < (n - 1); i++) {
      q = p[i * 2] * p[i * 2 + 3] - p[i * 2 + 2] * p[i * 2 + 1];
      a += q;
      cx += q * (p[i * 2] + p[i * 2 + 2]);
      cy += q * (p[i * 2 + 1] + p[i * 2 + 3]);
    }
    q = p[n * 2 - 2] * p[1] - p[0] * p[n * 2 - 1];
    a = 1.0 / (3.0 * (a + q));
    cx = a * (cx + q * (p[n * 2 - 2] + p[0]));
    cy = a * (cy + q * (p[n * 2 - 1] + p[1]));
  }
  real A[8];
  for (i = 0; i < n; i++) A[i] = atan2(p[i * 2 + 1] - cy, p[i * 2] - cx);
  int avail[8];
  for (i = 0; i < n; i++) avail[i] = 1;
  avail[i0] = 0;
  iret[0] = i0;
  iret++;
  for (j = 1; j < m; j++) {
    a = (real)((real)j * (2 * R_PI / m) + A[i0]);
    if (a > R_PI) a -= (real)(2 * R_PI);
    real maxdiff = 1e9, diff;
    for (i = 0; i < n; i++) {
      if (avail[i]) {
        diff = fabs(A[i] - a);
        if (diff > R_PI) diff = (real)(2 * R_PI - diff);
        if (diff < maxdiff) { maxdiff = diff; *iret = i; }
      }
    }
    avail[*iret] = 0;
    iret++;
  }
}

#define CONTACTS_UNIMPORTANT 0x80000000u

/* dBoxBox, ode/src/box.cpp:331-713. Fills pos/depth; returns count. */
static int box_box(const real* p1, const real* R1, const real* side1, const real* p2, const real* R2,
                   const real* side2, real* normal, real* depth, int* return_code, unsigned flags,
                   OContact* contact) {
  const real fudge_factor = 1.05;
  real p[3], pp[3], normalC[3] = {0, 0, 0};
  const real* normalR = 0;
  real A[3], B[3], R11, R12, R13, R21, R22, R23, R31, R32, R33, Q11, Q12, Q13, Q21, Q22, Q23, Q31, Q32,
      Q33, s, s2, l, e1;
  int i, j, invert_normal, code;

  p[0] = p2[0] - p1[0]; p[1] = p2[1] - p1[1]; p[2] = p2[2] - p1[2];
  mul1_331(pp, R1, p);
  A[0] = side1[0] * 0.5; A[1] = side1[1] * 0.5; A[2] = side1[2] * 0.5;
  B[0] = side2[0] * 0.5; B[1] = side2[1] * 0.5; B[2] = side2[2] * 0.5;

  R11 = dot3s(R1 + 0, R2 + 0, 4, 4); R12 = dot3s(R1 + 0, R2 + 1, 4, 4); R13 = dot3s(R1 + 0, R2 + 2, 4, 4);
  R21 = dot3s(R1 + 1, R2 + 0, 4, 4); R22 = dot3s(R1 + 1, R2 + 1, 4, 4); R23 = dot3s(R1 + 1, R2 + 2, 4, 4);
  R31 = dot3s(R1 + 2, R2 + 0, 4, 4); R32 = dot3s(R1 + 2, R2 + 1, 4, 4); R33 = dot3s(R1 + 2, R2 + 2, 4, 4);
  Q11 = fabs(R11); Q12 = fabs(R12); Q13 = fabs(R13);
  Q21 = fabs(R21); Q22 = fabs(R22); Q23 = fabs(R23);
  Q31 = fabs(R31); Q32 = fabs(R32); Q33 = fabs(R33);

  s = -R_INF;
  invert_normal = 0;
  code = 0;
  do {
#define TST_FACE(expr1, expr2, norm, cc)          \
  e1 = (expr1);                                   \
  s2 = fabs(e1) - (expr2);                        \
  if (s2 > 0) return 0;                           \
  if (s2 > s) {                                   \
    s = s2; normalR = norm; invert_normal = (e1 < 0); code = (cc); \
    if (flags & CONTACTS_UNIMPORTANT) break;      \
  }
    TST_FACE(pp[0], (A[0] + B[0] * Q11 + B[1] * Q12 + B[2] * Q13), R1 + 0, 1);
    TST_FACE(pp[1], (A[1] + B[0] * Q21 + B[1] * Q22 + B[2] * Q23), R1 + 1, 2);
    TST_FACE(pp[2], (A[2] + B[0] * Q31 + B[1] * Q32 + B[2] * Q33), R1 + 2, 3);
    TST_FACE(dot3s(R2 + 0, p, 4, 1), (A[0] * Q11 + A[1] * Q21 + A[2] * Q31 + B[0]), R2 + 0, 4);
    TST_FACE(dot3s(R2 + 1, p, 4, 1), (A[0] * Q12 + A[1] * Q22 + A[2] * Q32 + B[1]), R2 + 1, 5);
    TST_FACE(dot3s(R2 + 2, p, 4, 1), (A[0] * Q13 + A[1] * Q23 + A[2] * Q33 + B[2]), R2 + 2, 6);
#undef TST_FACE
#define TST_EDGE(expr1, expr2, n1, n2, n3, cc)              \
  e1 = (expr1);                                             \
  s2 = fabs(e1) - (expr2);                                  \
  if (s2 > 0) return 0;                                     \
  l = sqrt((n1) * (n1) + (n2) * (n2) + (n3) * (n3));        \
  if (l > 0) {                                              \
    s2 /= l;                                                \
    if (s2 * fudge_factor > s) {                            \
      s = s2; normalR = 0;                                  \
      normalC[0] = (n1) / l; normalC[1] = (n2) / l; normalC[2] = (n3) / l; \
      invert_normal = (e1 < 0); code = (cc);                \
      if (flags & CONTACTS_UNIMPORTANT) break;              \
    }                                                       \
  }
    TST_EDGE(pp[2] * R21 - pp[1] * R31, (A[1] * Q31 + A[2] * Q21 + B[1] * Q13 + B[2] * Q12), 0, -R31, R21, 7);
    TST_EDGE(pp[2] * R22 - pp[1] * R32, (A[1] * Q32 + A[2] * Q22 + B[0] * Q13 + B[2] * Q11), 0, -R32, R22, 8);
    TST_EDGE(pp[2] * R23 - pp[1] * R33, (A[1] * Q33 + A[2] * Q23 + B[0] * Q12 + B[1] * Q11), 0, -R33, R23, 9);
    TST_EDGE(pp[0] * R31 - pp[2] * R11, (A[0] * Q31 + A[2] * Q11 + B[1] * Q23 + B[2] * Q22), R31, 0, -R11, 10);
    TST_EDGE(pp[0] * R32 - pp[2] * R12, (A[0] * Q32 + A[2] * Q12 + B[0] * Q23 + B[2] * Q21), R32, 0, -R12, 11);
    TST_EDGE(pp[0] * R33 - pp[2] * R13, (A[0] * Q33 + A[2] * Q13 + B[0] * Q22 + B[1] * Q21), R33, 0, -R13, 12);
    TST_EDGE(pp[1] * R11 - pp[0] * R21, (A[0] * Q21 + A[1] * Q11 + B[1] * Q33 + B[2] * Q32), -R21, R11, 0, 13);
    TST_EDGE(pp[1] * R12 - pp[0] * R22, (A[0] * Q22 + A[1] * Q12 + B[0] * Q33 + B[2] * Q31), -R22, R12, 0, 14);
    TST_EDGE(pp[1] * R13 - pp[0] * R23, (A[0] * Q23 + A[1] * Q13 + B[0] * Q32 + B[1] * Q31), -R23, R13, 0, 15);
#undef TST_EDGE
  } while (0);

  if (!code) return 0;

  if (normalR) {
    normal[0] = normalR[0]; normal[1] = normalR[4]; normal[2] = normalR[8];
  } else {
    mul0_331(normal, R1, normalC);
  }
  if (invert_normal) { normal[0] = -normal[0]; normal[1] = -normal[1]; normal[2] = -normal[2]; }
  *depth = -s;

  if (code > 6) {
    real pa[3], pb[3], sign, alpha, beta, ua[3], ub[3];
    for (i = 0; i < 3; i++) pa[i] = p1[i];
    for (j = 0; j < 3; j++) {
      sign = (dot3s(normal, R1 + j, 1, 4) > 0) ? 1.0 : -1.0;
      for (i = 0; i < 3; i++) pa[i] += sign * A[j] * R1[i * 4 + j];
    }
    for (i = 0; i < 3; i++) pb[i] = p2[i];
    for (j = 0; j < 3; j++) {
      sign = (dot3s(normal, R2 + j, 1, 4) > 0) ? -1.0 : 1.0;
      for (i = 0; i < 3; i++) pb[i] += sign * B[j] * R2[i * 4 + j];
    }
    for (i = 0; i < 3; i++) ua[i] = R1[((code)-7) / 3 + i * 4];
    for (i = 0; i < 3; i++) ub[i] = R2[((code)-7) % 3 + i * 4];
    line_closest_approach(pa, ua, pb, ub, &alpha, &beta);
    for (i = 0; i < 3; i++) pa[i] += ua[i] * alpha;
    for (i = 0; i < 3; i++) pb[i] += ub[i] * beta;
    for (i = 0; i < 3; i++) contact[0].pos[i] = 0.5 * (pa[i] + pb[i]);
    contact[0].depth = *depth;
    *return_code = code;
    return 1;
  }

  const real *Ra, *Rb, *pa, *pb, *Sa, *Sb;
  if (code <= 3) { Ra = R1; Rb = R2; pa = p1; pb = p2; Sa = A; Sb = B; }
  else { Ra = R2; Rb = R1; pa = p2; pb = p1; Sa = B; Sb = A; }

  real normal2[3], nr[3], anr[3];
  if (code <= 3) { normal2[0] = normal[0]; normal2[1] = normal[1]; normal2[2] = normal[2]; }
  else { normal2[0] = -normal[0]; normal2[1] = -normal[1]; normal2[2] = -normal[2]; }
  mul1_331(nr, Rb, normal2);
  anr[0] = fabs(nr[0]); anr[1] = fabs(nr[1]); anr[2] = fabs(nr[2]);

  int lanr, a1, a2;
  if (anr[1] > anr[0]) {
    if (anr[1] > anr[2]) { a1 = 0; lanr = 1; a2 = 2; }
    else { a1 = 0; a2 = 1; lanr = 2; }
  } else {
    if (anr[0] > anr[2]) { lanr = 0; a1 = 1; a2 = 2; }
    else { a1 = 0; a2 = 1; lanr = 2; }
  }

  real center[3];
  if (nr[lanr] < 0) {
    for (i = 0; i < 3; i++) center[i] = pb[i] - pa[i] + Sb[lanr] * Rb[i * 4 + lanr];
  } else {
    for (i = 0; i < 3; i++) center[i] = pb[i] - pa[i] - Sb[lanr] * Rb[i * 4 + lanr];
  }

  int codeN, code1, code2;
  if (code <= 3) codeN = code - 1; else codeN = code - 4;
  if (codeN == 0) { code1 = 1; code2 = 2; }
  else if (codeN == 1) { code1 = 0; code2 = 2; }
  else { code1 = 0; code2 = 1; }

  real quad[8], c1, c2, m11, m12, m21, m22;
  c1 = dot3s(center, Ra + code1, 1, 4);
  c2 = dot3s(center, Ra + code2, 1, 4);
  m11 = dot3s(Ra + code1, Rb + a1, 4, 4);
  m12 = dot3s(Ra + code1, Rb + a2, 4, 4);
  m21 = dot3s(Ra + code2, Rb + a1, 4, 4);
  m22 = dot3s(Ra + code2, Rb + a2, 4, 4);
  {
    real k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
    quad[0] = c1 - k1 - k3; quad[1] = c2 - k2 - k4;
    quad[2] = c1 - k1 + k3; quad[3] = c2 - k2 + k4;
    quad[4] = c1 + k1 + k3; quad[5] = c2 + k2 + k4;
    quad[6] = c1 + k1 - k3; quad[7] = c2 + k2 - k4;
  }
  real rect[2] = {Sa[code1], Sa[code2]};
  real ret[16];
  int n = intersect_rect_quad(rect, quad, ret);
  if (n < 1) return 0;

  real point[3 * 8], dep[8];
  real det1 = 1.0 / (m11 * m22 - m12 * m21);
  m11 *= det1; m12 *= det1; m21 *= det1; m22 *= det1;
  int cnum = 0;
  for (j = 0; j < n; j++) {
    real k1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
    real k2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
    for (i = 0; i < 3; i++) point[cnum * 3 + i] = center[i] + k1 * Rb[i * 4 + a1] + k2 * Rb[i * 4 + a2];
    dep[cnum] = Sa[codeN] - dot3(normal2, point + cnum * 3);
    if (dep[cnum] >= 0) {
      ret[cnum * 2] = ret[j * 2];
      ret[cnum * 2 + 1] = ret[j * 2 + 1];
      cnum++;
      if ((cnum | CONTACTS_UNIMPORTANT) == (flags & (0xffffu | CONTACTS_UNIMPORTANT))) break;
    }
  }
  if (cnum < 1) return 0;

  int maxc = flags & 0xffff;
  if (maxc > cnum) maxc = cnum;
  if (maxc < 1) maxc = 1;
  if (cnum <= maxc) {
    for (j = 0; j < cnum; j++) {
      for (i = 0; i < 3; i++) contact[j].pos[i] = point[j * 3 + i] + pa[i];
      contact[j].depth = dep[j];
    }
  } else {
    int i1 = 0;
    real maxdepth = dep[0];
    for (i = 1; i < cnum; i++) {
      if (dep[i] > maxdepth) { maxdepth = dep[i]; i1 = i; }
    }
    int iret[8];
    cull_points(cnum, ret, maxc, i1, iret);
    for (j = 0; j < maxc; j++) {
      for (i = 0; i < 3; i++) contact[j].pos[i] = point[iret[j] * 3 + i] + pa[i];
      contact[j].depth = dep[iret[j]];
    }
    cnum = maxc;
  }
  *return_code = code;
  return cnum;
}

/* dCollideBoxBox, ode/src/box.cpp:716-742 (normal negated) */
static int collide_box_box(const GeomRef* a, const GeomRef* b, unsigned flags, OContact* c) {
  real normal[3], depth;
  int code;
  int num = box_box(a->pos, a->R, a->p, b->pos, b->R, b->p, normal, &depth, &code, flags, c);
  for (int i = 0; i < num; i++) {
    c[i].normal[0] = -normal[0]; c[i].normal[1] = -normal[1]; c[i].normal[2] = -normal[2];
  }
  return num;
}

/* dCollideBoxPlane, ode/src/box.cpp:745-878 */
static int collide_box_plane(const GeomRef* bx, const GeomRef* pl, unsigned flags, OContact* c) {
  const real* R = bx->R;
  const real* n = pl->p;
  const real* side = bx->p;
  real Q1 = dot3s(n, R + 0, 1, 4), Q2 = dot3s(n, R + 1, 1, 4), Q3 = dot3s(n, R + 2, 1, 4);
  real A1 = side[0] * Q1, A2 = side[1] * Q2, A3 = side[2] * Q3;
  real B1 = fabs(A1), B2 = fabs(A2), B3 = fabs(A3);
  real depth = n[3] + 0.5 * (B1 + B2 + B3) - dot3(n, bx->pos);
  if (depth < 0) return 0;
  int maxc = flags & 0xffff;
  if (maxc > 4) maxc = 4;
  real p[3] = {bx->pos[0], bx->pos[1], bx->pos[2]};
  real Aarr[3] = {A1, A2, A3};
  for (int i = 0; i < 3; ++i) {
    if (Aarr[i] > 0) {
      p[0] -= 0.5 * side[i] * R[0 + i]; p[1] -= 0.5 * side[i] * R[4 + i]; p[2] -= 0.5 * side[i] * R[8 + i];
    } else {
      p[0] += 0.5 * side[i] * R[0 + i]; p[1] += 0.5 * side[i] * R[4 + i]; p[2] += 0.5 * side[i] * R[8 + i];
    }
  }
  c[0].pos[0] = p[0]; c[0].pos[1] = p[1]; c[0].pos[2] = p[2];
  c[0].depth = depth;
  int ret = 1;
  real Barr[3] = {B1, B2, B3};
  /* add contact `ct` by walking from p along side `sd` (0-based) */
#define ADD_SIDE(ct, sd)                                                    \
  do {                                                                      \
    if (depth - Barr[sd] < 0) goto done;                                    \
    if (Aarr[sd] > 0) {                                                     \
      c[ct].pos[0] = p[0] + side[sd] * R[0 + sd];                           \
      c[ct].pos[1] = p[1] + side[sd] * R[4 + sd];                           \
      c[ct].pos[2] = p[2] + side[sd] * R[8 + sd];                           \
    } else {                                                                \
      c[ct].pos[0] = p[0] - side[sd] * R[0 + sd];                           \
      c[ct].pos[1] = p[1] - side[sd] * R[4 + sd];                           \
      c[ct].pos[2] = p[2] - side[sd] * R[8 + sd];                           \
    }                                                                       \
    c[ct].depth = depth - Barr[sd];                                         \
    ret++;                                                                  \
  } while (0)
  if (maxc == 1) goto done;
  if (B1 < B2) {
    if (B3 < B1) goto use_side_3;
    ADD_SIDE(1, 0);
    if (maxc == 2) goto done;
    if (B2 < B3) goto contact2_2; else goto contact2_3;
  } else {
    if (B3 < B2) {
    use_side_3:
      ADD_SIDE(1, 2);
      if (maxc == 2) goto done;
      if (B1 < B2) goto contact2_1; else goto contact2_2;
    } else {
      ADD_SIDE(1, 1);
      if (maxc == 2) goto done;
      if (B1 < B3) goto contact2_1; else goto contact2_3;
    }
  }
contact2_1: ADD_SIDE(2, 0); goto done;
contact2_2: ADD_SIDE(2, 1); goto done;
contact2_3: ADD_SIDE(2, 2); goto done;
#undef ADD_SIDE
done:
  if (maxc == 4 && ret == 3) {
    real d4 = c[1].depth + c[2].depth - depth;
    if (d4 > 0) {
      c[3].pos[0] = c[1].pos[0] + c[2].pos[0] - p[0];
      c[3].pos[1] = c[1].pos[1] + c[2].pos[1] - p[1];
      c[3].pos[2] = c[1].pos[2] + c[2].pos[2] - p[2];
      c[3].depth = d4;
      ret++;
    }
  }
  for (int i = 0; i < ret; i++) {
    c[i].normal[0] = n[0]; c[i].normal[1] = n[1]; c[i].normal[2] = n[2];
  }
  return ret;
}

/* dCollideCapsulePlane, ode/src/capsule.cpp:352-411 */
static int collide_capsule_plane(const GeomRef* cp, const GeomRef* pl, unsigned flags, OContact* c) {
  const real* R = cp->R;
  const real* P = pl->p;
  real radius = cp->p[0], lz = cp->p[1];
  real sign = (dot3s(P, R + 2, 1, 4) > 0) ? -1.0 : 1.0;
  real p[3];
  p[0] = cp->pos[0] + R[2] * lz * 0.5 * sign;
  p[1] = cp->pos[1] + R[6] * lz * 0.5 * sign;
  p[2] = cp->pos[2] + R[10] * lz * 0.5 * sign;
  real k = dot3(p, P);
  real depth = P[3] - k + radius;
  if (depth < 0) return 0;
  c[0].normal[0] = P[0]; c[0].normal[1] = P[1]; c[0].normal[2] = P[2];
  c[0].pos[0] = p[0] - P[0] * radius;
  c[0].pos[1] = p[1] - P[1] * radius;
  c[0].pos[2] = p[2] - P[2] * radius;
  c[0].depth = depth;
  int nc = 1;
  if ((flags & 0xffff) >= 2) {
    p[0] = cp->pos[0] - R[2] * lz * 0.5 * sign;
    p[1] = cp->pos[1] - R[6] * lz * 0.5 * sign;
    p[2] = cp->pos[2] - R[10] * lz * 0.5 * sign;
    k = dot3(p, P);
    depth = P[3] - k + radius;
    if (depth >= 0) {
      c[1].normal[0] = P[0]; c[1].normal[1] = P[1]; c[1].normal[2] = P[2];
      c[1].pos[0] = p[0] - P[0] * radius;
      c[1].pos[1] = p[1] - P[1] * radius;
      c[1].pos[2] = p[2] - P[2] * radius;
      c[1].depth = depth;
      nc = 2;
    }
  }
  return nc;
}

/* dCollideCapsuleSphere, ode/src/capsule.cpp:130-160 */
static int collide_capsule_sphere(const GeomRef* cp, const GeomRef* sp, OContact* c) {
  const real* R = cp->R;
  real alpha = R[2] * (sp->pos[0] - cp->pos[0]) + R[6] * (sp->pos[1] - cp->pos[1]) +
               R[10] * (sp->pos[2] - cp->pos[2]);
  const real lz2 = cp->p[1] * 0.5;
  if (alpha > lz2) alpha = lz2;
  if (alpha < -lz2) alpha = -lz2;
  real p[3] = {cp->pos[0] + alpha * R[2], cp->pos[1] + alpha * R[6], cp->pos[2] + alpha * R[10]};
  return collide_spheres(p, cp->p[0], sp->pos, sp->p[0], c);
}

/* dCollideSpheresZeroDist, ode/src/capsule.cpp:164-176 */
static int collide_spheres_zero_dist(const real* p1, real r1, real r2, const real* normal, OContact* c) {
  c->normal[0] = normal[0]; c->normal[1] = normal[1]; c->normal[2] = normal[2];
  c->depth = r1 + r2;
  const real k = 0.5 * (r2 - r1);
  c->pos[0] = p1[0] + c->normal[0] * k;
  c->pos[1] = p1[1] + c->normal[1] * k;
  c->pos[2] = p1[2] + c->normal[2] * k;
  return 1;
}

/* dClosestLineBoxPoints, ode/src/collision_util.cpp:247-372 (dDOUBLE) */
static void closest_line_box_points(const real* p1, const real* p2, const real* c, const real* R,
                                    const real* side, real* lret, real* bret) {
  real tmp[3], s[3], v[3], sign[3], v2[3], h[3], tanchor[3];
  int region[3];
  tmp[0] = p1[0] - c[0]; tmp[1] = p1[1] - c[1]; tmp[2] = p1[2] - c[2];
  mul1_331(s, R, tmp);
  tmp[0] = p2[0] - p1[0]; tmp[1] = p2[1] - p1[1]; tmp[2] = p2[2] - p1[2];
  mul1_331(v, R, tmp);
  for (int i = 0; i < 3; i++) {
    if (v[i] < 0) { s[i] = -s[i]; v[i] = -v[i]; sign[i] = -1; }
    else sign[i] = 1;
  }
  for (int i = 0; i < 3; i++) v2[i] = v[i] * v[i];
  for (int i = 0; i < 3; i++) h[i] = 0.5 * side[i];
  const real tanchor_eps = 1e-307;
  for (int i = 0; i < 3; i++) {
    if (v[i] > tanchor_eps) {
      if (s[i] < -h[i]) { region[i] = -1; tanchor[i] = (-h[i] - s[i]) / v[i]; }
      else { region[i] = (s[i] > h[i]); tanchor[i] = (h[i] - s[i]) / v[i]; }
    } else {
      region[i] = 0;
      tanchor[i] = 2;
    }
  }
  real t = 0, dd2dt = 0;
  for (int i = 0; i < 3; i++) dd2dt -= (region[i] ? v2[i] : 0) * tanchor[i];
  if (dd2dt >= 0) goto got_answer;
  do {
    real next_t = 1;
    for (int i = 0; i < 3; i++)
      if (tanchor[i] > t && tanchor[i] < 1 && tanchor[i] < next_t) next_t = tanchor[i];
    real next_dd2dt = 0;
    for (int i = 0; i < 3; i++) next_dd2dt += (region[i] ? v2[i] : 0) * (next_t - tanchor[i]);
    if (next_dd2dt >= 0) {
      const real m = (next_dd2dt - dd2dt) / (next_t - t);
      t -= dd2dt / m;
      goto got_answer;
    }
    for (int i = 0; i < 3; i++) {
      if (tanchor[i] == next_t) {
        tanchor[i] = (h[i] - s[i]) / v[i];
        region[i]++;
      }
    }
    t = next_t;
    dd2dt = next_dd2dt;
  } while (t < 1);
  t = 1;
got_answer:
  for (int i = 0; i < 3; i++) lret[i] = p1[i] + t * tmp[i];
  for (int i = 0; i < 3; i++) {
    tmp[i] = sign[i] * (s[i] + t * v[i]);
    if (tmp[i] < -h[i]) tmp[i] = -h[i];
    else if (tmp[i] > h[i]) tmp[i] = h[i];
  }
  mul0_331(s, R, tmp);
  for (int i = 0; i < 3; i++) bret[i] = s[i] + c[i];
}

/* dClosestLineSegmentPoints, ode/src/collision_util.cpp:109-209 */
static void closest_segment_points(const real* a1, const real* a2, const real* b1, const real* b2, real* cp1,
                                   real* cp2) {
  real a1a2[3], b1b2[3], a1b1[3], a1b2[3], a2b1[3], a2b2[3], n[3];
  for (int i = 0; i < 3; ++i) { a1a2[i] = a2[i] - a1[i]; b1b2[i] = b2[i] - b1[i]; a1b1[i] = b1[i] - a1[i]; }
  const real da1 = dot3(a1a2, a1b1), db1 = dot3(b1b2, a1b1);
  if (da1 <= 0 && db1 >= 0) { for (int i = 0; i < 3; ++i) { cp1[i] = a1[i]; cp2[i] = b1[i]; } return; }
  for (int i = 0; i < 3; ++i) a1b2[i] = b2[i] - a1[i];
  const real da2 = dot3(a1a2, a1b2), db2 = dot3(b1b2, a1b2);
  if (da2 <= 0 && db2 <= 0) { for (int i = 0; i < 3; ++i) { cp1[i] = a1[i]; cp2[i] = b2[i]; } return; }
  for (int i = 0; i < 3; ++i) a2b1[i] = b1[i] - a2[i];
  const real da3 = dot3(a1a2, a2b1), db3 = dot3(b1b2, a2b1);
  if (da3 >= 0 && db3 >= 0) { for (int i = 0; i < 3; ++i) { cp1[i] = a2[i]; cp2[i] = b1[i]; } return; }
  for (int i = 0; i < 3; ++i) a2b2[i] = b2[i] - a2[i];
  const real da4 = dot3(a1a2, a2b2), db4 = dot3(b1b2, a2b2);
  if (da4 >= 0 && db4 <= 0) { for (int i = 0; i < 3; ++i) { cp1[i] = a2[i]; cp2[i] = b2[i]; } return; }
  const real la = dot3(a1a2, a1a2);
  if (da1 >= 0 && da3 <= 0) {
    const real k = da1 / la;
    for (int i = 0; i < 3; ++i) n[i] = a1b1[i] - k * a1a2[i];
    if (dot3(b1b2, n) >= 0) {
      for (int i = 0; i < 3; ++i) { cp1[i] = a1[i] + k * a1a2[i]; cp2[i] = b1[i]; }
      return;
    }
  }
  if (da2 >= 0 && da4 <= 0) {
    const real k = da2 / la;
    for (int i = 0; i < 3; ++i) n[i] = a1b2[i] - k * a1a2[i];
    if (dot3(b1b2, n) <= 0) {
      for (int i = 0; i < 3; ++i) { cp1[i] = a1[i] + k * a1a2[i]; cp2[i] = b2[i]; }
      return;
    }
  }
  const real lb = dot3(b1b2, b1b2);
  if (db1 <= 0 && db2 >= 0) {
    const real k = -db1 / lb;
    for (int i = 0; i < 3; ++i) n[i] = -a1b1[i] - k * b1b2[i];
    if (dot3(a1a2, n) >= 0) {
      for (int i = 0; i < 3; ++i) { cp1[i] = a1[i]; cp2[i] = b1[i] + k * b1b2[i]; }
      return;
    }
  }
  if (db3 <= 0 && db4 >= 0) {
    const real k = -db3 / lb;
    for (int i = 0; i < 3; ++i) n[i] = -a2b1[i] - k * b1b2[i];
    if (dot3(a1a2, n) <= 0) {
      for (int i = 0; i < 3; ++i) { cp1[i] = a2[i]; cp2[i] = b1[i] + k * b1b2[i]; }
      return;
    }
  }
  const real k = dot3(a1a2, b1b2);
  real det = la * lb - k * k;
  if (det <= 0) { for (int i = 0; i < 3; ++i) { cp1[i] = a1[i]; cp2[i] = b1[i]; } return; }
  det = 1.0 / det;
  const real alpha = (lb * da1 - k * db1) * det;
  const real beta = (k * da1 - la * db1) * det;
  for (int i = 0; i < 3; ++i) { cp1[i] = a1[i] + alpha * a1a2[i]; cp2[i] = b1[i] + beta * b1b2[i]; }
}

/* dCollideCapsuleBox, ode/src/capsule.cpp:178-229 */
static int collide_capsule_box(const GeomRef* cp, const GeomRef* bx, OContact* c) {
  const real* R1 = cp->R;
  const real clen = cp->p[1] * 0.5;
  real p1[3], p2[3], pl[3], pb[3];
  for (int i = 0; i < 3; ++i) {
    p1[i] = cp->pos[i] + clen * R1[4 * i + 2];
    p2[i] = cp->pos[i] - clen * R1[4 * i + 2];
  }
  closest_line_box_points(p1, p2, bx->pos, bx->R, bx->p, pl, pb);
  const real mindist = 1e-18;
  const real dx = pl[0] - pb[0], dy = pl[1] - pb[1], dz = pl[2] - pb[2];
  if (sqrt(dx * dx + dy * dy + dz * dz) < mindist) {
    real normal[3] = {pb[0] - bx->pos[0], pb[1] - bx->pos[1], pb[2] - bx->pos[2]};
    safe_normalize3(normal);
    return collide_spheres_zero_dist(pl, cp->p[0], 0, normal, c);
  }
  return collide_spheres(pl, cp->p[0], pb, 0, c);
}

/* dCollideCapsuleCapsule, ode/src/capsule.cpp:232-350 */
static int collide_capsule_capsule(const GeomRef* g1, const GeomRef* g2, unsigned flags, OContact* c) {
  const real tolerance = 1e-5;
  const real lz1 = g1->p[1] * 0.5, lz2 = g2->p[1] * 0.5;
  const real* pos1 = g1->pos;
  const real* pos2 = g2->pos;
  real axis1[3] = {g1->R[2], g1->R[6], g1->R[10]};
  real axis2[3] = {g2->R[2], g2->R[6], g2->R[10]};
  real sphere1[3], sphere2[3];
  const real a1a2 = dot3(axis1, axis2);
  const real det = 1.0 - a1a2 * a1a2;
  if (det < tolerance) {
    if (a1a2 < 0) { axis2[0] = -axis2[0]; axis2[1] = -axis2[1]; axis2[2] = -axis2[2]; }
    real q[3];
    for (int i = 0; i < 3; i++) q[i] = pos1[i] - pos2[i];
    const real k = dot3(axis1, q);
    const real a1lo = -lz1, a1hi = lz1, a2lo = -lz2 - k, a2hi = lz2 - k;
    const real lo = (a1lo > a2lo) ? a1lo : a2lo;
    const real hi = (a1hi < a2hi) ? a1hi : a2hi;
    if (lo <= hi) {
      const int num_contacts = (int)(flags & 0xffff);
      if (num_contacts >= 2 && lo < hi) {
        for (int i = 0; i < 3; i++) sphere1[i] = pos1[i] + lo * axis1[i];
        for (int i = 0; i < 3; i++) sphere2[i] = pos2[i] + (lo + k) * axis2[i];
        const int n1 = collide_spheres(sphere1, g1->p[0], sphere2, g2->p[0], c);
        if (n1) {
          for (int i = 0; i < 3; i++) sphere1[i] = pos1[i] + hi * axis1[i];
          for (int i = 0; i < 3; i++) sphere2[i] = pos2[i] + (hi + k) * axis2[i];
          const int n2 = collide_spheres(sphere1, g1->p[0], sphere2, g2->p[0], c + 1);
          if (n2) return 2;
        }
      }
      const real alpha1 = (lo + hi) * 0.5;
      const real alpha2 = alpha1 + k;
      for (int i = 0; i < 3; i++) sphere1[i] = pos1[i] + alpha1 * axis1[i];
      for (int i = 0; i < 3; i++) sphere2[i] = pos2[i] + alpha2 * axis2[i];
      return collide_spheres(sphere1, g1->p[0], sphere2, g2->p[0], c);
    }
  }
  real a1[3], a2[3], b1[3], b2[3];
  for (int i = 0; i < 3; ++i) {
    a1[i] = pos1[i] + axis1[i] * lz1;
    a2[i] = pos1[i] - axis1[i] * lz1;
    b1[i] = pos2[i] + axis2[i] * lz2;
    b2[i] = pos2[i] - axis2[i] * lz2;
  }
  closest_segment_points(a1, a2, b1, b2, sphere1, sphere2);
  return collide_spheres(sphere1, g1->p[0], sphere2, g2->p[0], c);
}

/* ---- rays (ode/src/ray.cpp). A ray geom holds its length in p[0]; it starts
 * at pos and points along column 2 of R (dGeomRaySet, ray.cpp:115-136). Each
 * ray collider returns at most one contact whose depth is the distance from
 * the ray's start along the ray. */

/* ray_sphere_helper, ray.cpp:196-233: mode 1 takes the exit point. */
static int ray_sphere_helper(const GeomRef* ray, const real* spos, real radius, OContact* c, int mode) {
  const real* rp = ray->pos;
  const real* R = ray->R;
  const real q[3] = {rp[0] - spos[0], rp[1] - spos[1], rp[2] - spos[2]};
  const real B = q[0] * R[2] + q[1] * R[6] + q[2] * R[10];
  const real C = dot3(q, q) - radius * radius;
  real k = B * B - C;
  if (k < 0) return 0;
  k = sqrt(k);
  real alpha;
  if (mode && C >= 0) {
    alpha = -B + k;
    if (alpha < 0) return 0;
  } else {
    alpha = -B - k;
    if (alpha < 0) {
      alpha = -B + k;
      if (alpha < 0) return 0;
    }
  }
  if (alpha > ray->p[0]) return 0;
  for (int i = 0; i < 3; ++i) c->pos[i] = rp[i] + alpha * R[i * 4 + 2];
  const real nsign = (C < 0 || mode) ? -1.0 : 1.0;
  for (int i = 0; i < 3; ++i) c->normal[i] = nsign * (c->pos[i] - spos[i]);
  safe_normalize3(c->normal);
  c->depth = alpha;
  return 1;
}

/* dCollideRaySphere, ray.cpp:235-251 */
static int collide_ray_sphere(const GeomRef* ray, const GeomRef* s, OContact* c) {
  return ray_sphere_helper(ray, s->pos, s->p[0], c, 0);
}

/* dCollideRayBox, ray.cpp:253-350: slab test in the box frame with the ray
 * mirrored so that its direction has no negative component. */
static int collide_ray_box(const GeomRef* ray, const GeomRef* bx, OContact* c) {
  const real* rp = ray->pos;
  const real* RR = ray->R;
  const real* BR = bx->R;
  real tmp[3] = {rp[0] - bx->pos[0], rp[1] - bx->pos[1], rp[2] - bx->pos[2]};
  real s[3], v[3], sign[3];
  mul1_331(s, BR, tmp);
  tmp[0] = RR[2]; tmp[1] = RR[6]; tmp[2] = RR[10];
  mul1_331(v, BR, tmp);
  for (int i = 0; i < 3; ++i) {
    if (v[i] < 0) { s[i] = -s[i]; v[i] = -v[i]; sign[i] = 1; }
    else sign[i] = -1;
  }
  const real h[3] = {0.5 * bx->p[0], 0.5 * bx->p[1], 0.5 * bx->p[2]};
  if ((s[0] < -h[0] && v[0] <= 0) || s[0] > h[0] || (s[1] < -h[1] && v[1] <= 0) || s[1] > h[1] ||
      (s[2] < -h[2] && v[2] <= 0) || s[2] > h[2] || (v[0] == 0 && v[1] == 0 && v[2] == 0))
    return 0;
  real lo = -INFINITY, hi = INFINITY;
  int nlo = 0, nhi = 0;
  for (int i = 0; i < 3; ++i) {
    if (v[i] != 0) {
      real k = (-h[i] - s[i]) / v[i];
      if (k > lo) { lo = k; nlo = i; }
      k = (h[i] - s[i]) / v[i];
      if (k < hi) { hi = k; nhi = i; }
    }
  }
  if (lo > hi) return 0;
  real alpha;
  int n;
  if (lo >= 0) { alpha = lo; n = nlo; }
  else { alpha = hi; n = nhi; }
  if (alpha < 0 || alpha > ray->p[0]) return 0;
  for (int i = 0; i < 3; ++i) {
    c->pos[i] = rp[i] + alpha * RR[i * 4 + 2];
    c->normal[i] = BR[i * 4 + n] * sign[n];
  }
  c->depth = alpha;
  return 1;
}

/* dCollideRayCapsule, ray.cpp:352-465: the infinite cylinder first, then the
 * cap sphere on the side the hit (or the start) lies. */
static int collide_ray_capsule(const GeomRef* ray, const GeomRef* cp, OContact* c) {
  const real* rp = ray->pos;
  const real* RR = ray->R;
  const real* CR = cp->R;
  const real* cpos = cp->pos;
  const real radius = cp->p[0];
  const real lz2 = cp->p[1] * 0.5;
  const real cs[3] = {rp[0] - cpos[0], rp[1] - cpos[1], rp[2] - cpos[2]};
  real k = CR[2] * cs[0] + CR[6] * cs[1] + CR[10] * cs[2];
  real q[3], r[3];
  for (int i = 0; i < 3; ++i) q[i] = k * CR[i * 4 + 2] - cs[i];
  real C = dot3(q, q) - radius * radius;
  int inside = 0;
  if (C < 0) {
    if (k < -lz2) k = -lz2;
    else if (k > lz2) k = lz2;
    for (int i = 0; i < 3; ++i) r[i] = cpos[i] + k * CR[i * 4 + 2];
    if ((rp[0] - r[0]) * (rp[0] - r[0]) + (rp[1] - r[1]) * (rp[1] - r[1]) + (rp[2] - r[2]) * (rp[2] - r[2]) <
        radius * radius)
      inside = 1;
  }
  if (!inside && C < 0) {
    k = (k < 0) ? -lz2 : lz2;
  } else {
    const real uv = CR[2] * RR[2] + CR[6] * RR[6] + CR[10] * RR[10];
    for (int i = 0; i < 3; ++i) r[i] = uv * CR[i * 4 + 2] - RR[i * 4 + 2];
    real A = dot3(r, r);
    const real B = 2 * dot3(q, r);
    k = B * B - 4 * A * C;
    if (k < 0) {
      if (!inside) return 0;
      k = (uv < 0) ? -lz2 : lz2;
    } else {
      k = sqrt(k);
      A = 1.0 / (2 * A);
      real alpha = (-B - k) * A;
      if (alpha < 0) {
        alpha = (-B + k) * A;
        if (alpha < 0) return 0;
      }
      if (alpha > ray->p[0]) return 0;
      for (int i = 0; i < 3; ++i) c->pos[i] = rp[i] + alpha * RR[i * 4 + 2];
      for (int i = 0; i < 3; ++i) q[i] = c->pos[i] - cpos[i];
      k = q[0] * CR[2] + q[1] * CR[6] + q[2] * CR[10];
      const real nsign = inside ? -1.0 : 1.0;
      if (k >= -lz2 && k <= lz2) {
        for (int i = 0; i < 3; ++i) c->normal[i] = nsign * (c->pos[i] - (cpos[i] + k * CR[i * 4 + 2]));
        safe_normalize3(c->normal);
        c->depth = alpha;
        return 1;
      }
      k = (k < 0) ? -lz2 : lz2;
    }
  }
  for (int i = 0; i < 3; ++i) q[i] = cpos[i] + k * CR[i * 4 + 2];
  return ray_sphere_helper(ray, q, radius, c, inside);
}

/* dCollideRayPlane, ray.cpp:467-498 */
static int collide_ray_plane(const GeomRef* ray, const GeomRef* pl, OContact* c) {
  const real* rp = ray->pos;
  const real* RR = ray->R;
  const real* P = pl->p;
  real alpha = P[3] - dot3(P, rp);
  const real nsign = (alpha > 0) ? -1.0 : 1.0;
  const real k = P[0] * RR[2] + P[1] * RR[6] + P[2] * RR[10];
  if (k == 0) return 0;
  alpha /= k;
  if (alpha < 0 || alpha > ray->p[0]) return 0;
  for (int i = 0; i < 3; ++i) {
    c->pos[i] = rp[i] + alpha * RR[i * 4 + 2];
    c->normal[i] = nsign * P[i];
  }
  c->depth = alpha;
  return 1;
}

/* ---- cylinders (flat-ended; ode/src/cylinder.cpp): p[0] radius, p[1] length
 * along column 2 of R. The dDOUBLE build's tolerance ("toleranz") is 1e-7. */
#define CYL_TOL 1e-7

/* dCollideCylinderSphere, ode/src/collision_cylinder_sphere.cpp:56-276: side,
 * disc or disc-rim contact from the sphere centre's axial (s) and radial (t)
 * distances. */
static int collide_cylinder_sphere(const GeomRef* cy, const GeomRef* sp, OContact* c) {
  const real radius = cy->p[0], length = cy->p[1];
  const real* cp = cy->pos;
  const real r2 = sp->p[0];
  const real* S = sp->pos;
  const real v[3] = {cy->R[2], cy->R[6], cy->R[10]};
  real s = length * 0.5;
  real P1[3], P2[3], C[3];
  for (int i = 0; i < 3; ++i) { P2[i] = v[i] * s + cp[i]; P1[i] = v[i] * -s + cp[i]; }
  s = (S[0] - P1[0]) * v[0] - (P1[1] - S[1]) * v[1] - (P1[2] - S[2]) * v[2];
  if (s < (-r2) || s > (length + r2)) return 0;
  for (int i = 0; i < 3; ++i) C[i] = s * v[i] + P1[i] - S[i];
  const real t = sqrt(dot3(C, C));
  if (t > (radius + r2)) return 0;
  if (t > radius && (s < 0 || s > length)) {
    const real* P = (s <= 0) ? P1 : P2;
    const real ds = (s <= 0) ? s : (s - length);
    c->depth = r2 - sqrt(ds * ds + (t - radius) * (t - radius));
    if (c->depth < 0) return 0;
    for (int i = 0; i < 3; ++i) c->pos[i] = C[i] / t * -radius + P[i];
    for (int i = 0; i < 3; ++i) c->normal[i] = (c->pos[i] - S[i]) / (r2 - c->depth);
    return 1;
  } else if ((radius - t) <= s && (radius - t) <= (length - s)) {
    c->depth = (r2 + radius) - t;
    if (c->depth < 0) return 0;
    if (t > (r2 + CYL_TOL)) {
      for (int i = 0; i < 3; ++i) C[i] /= t;
      for (int i = 0; i < 3; ++i) { c->pos[i] = C[i] * r2 + S[i]; c->normal[i] = C[i]; }
    } else {
      for (int i = 0; i < 3; ++i) { c->pos[i] = C[i] + S[i]; c->normal[i] = C[i] / t; }
    }
    return 1;
  }
  if (s <= (length * 0.5)) {
    c->depth = s + r2;
    if (c->depth < 0) return 0;
    for (int i = 0; i < 3; ++i) { c->pos[i] = r2 * v[i] + S[i]; c->normal[i] = v[i]; }
  } else {
    c->depth = (r2 + length - s);
    if (c->depth < 0) return 0;
    for (int i = 0; i < 3; ++i) { c->pos[i] = r2 * -v[i] + S[i]; c->normal[i] = -v[i]; }
  }
  return 1;
}

/* dCollideCylinderPlane, ode/src/collision_cylinder_plane.cpp:43-265: four rim
 * points of the lower disc when the axis is parallel to the plane normal, else
 * the deepest rim point of each disc. */
static int collide_cylinder_plane(const GeomRef* cy, const GeomRef* pl, unsigned flags, OContact* c) {
  const int maxc = (int)(flags & 0xffff);
  const real radius = cy->p[0], length = cy->p[1];
  const real* cp = cy->pos;
  const real* P = pl->p;
  const real v[3] = {cy->R[2], cy->R[6], cy->R[10]};
  real s = length * 0.5;
  real P1[3], P2[3];
  for (int i = 0; i < 3; ++i) { P2[i] = v[i] * s + cp[i]; P1[i] = v[i] * -s + cp[i]; }
  int n = 0;
  s = v[0] * P[0] + v[1] * P[1] + v[2] * P[2];
  if (s < 0) s += 1.0;
  else s -= 1.0;
  if (s < CYL_TOL && s > (-CYL_TOL)) {
    real Q[3];
    s = P[3] - dot3(P, P1);
    real t = P[3] - dot3(P, P2);
    if (s >= t) {
      if (s >= 0) { Q[0] = P1[0]; Q[1] = P1[1]; Q[2] = P1[2]; }
      else return 0;
    } else {
      if (t >= 0) { Q[0] = P2[0]; Q[1] = P2[1]; Q[2] = P2[2]; }
      else return 0;
    }
    real V1[3], V2[3];
    if (v[0] < CYL_TOL && v[0] > (-CYL_TOL)) { V1[0] = v[0] + 1.0; V1[1] = v[1]; V1[2] = v[2]; }
    else { V1[0] = v[0]; V1[1] = v[1] + 1.0; V1[2] = v[2]; }
    cross3(V2, V1, v);
    t = sqrt(dot3(V2, V2));
    t = radius / t;
    for (int i = 0; i < 3; ++i) V2[i] *= t;
    cross3(V1, V2, v);
    for (int k = 0; k < 4; ++k) {
      const real* A = (k < 2) ? V1 : V2;
      const real sg = (k & 1) ? -1.0 : 1.0;
      OContact* o = &c[n];
      for (int i = 0; i < 3; ++i) o->pos[i] = Q[i] + sg * A[i];
      o->depth = P[3] - dot3(P, o->pos);
      if (o->depth > 0) {
        o->normal[0] = P[0]; o->normal[1] = P[1]; o->normal[2] = P[2];
        if (++n >= maxc) return n;
      }
    }
  } else {
    const real t = dot3(P, v);
    real C[3];
    for (int i = 0; i < 3; ++i) C[i] = v[i] * t - P[i];
    s = sqrt(dot3(C, C));
    s = radius / s;
    for (int i = 0; i < 3; ++i) C[i] *= s;
    OContact* o = &c[n];
    for (int i = 0; i < 3; ++i) o->pos[i] = C[i] + P1[i];
    o->depth = P[3] - dot3(P, o->pos);
    if (o->depth >= 0) {
      o->normal[0] = P[0]; o->normal[1] = P[1]; o->normal[2] = P[2];
      if (++n >= maxc) return n;
    }
    o = &c[n];
    for (int i = 0; i < 3; ++i) o->pos[i] = C[i] + P2[i];
    o->depth = P[3] - P[0] * o->pos[0] - P[1] * o->pos[1] - P[2] * o->pos[2];
    if (o->depth >= 0) {
      o->normal[0] = P[0]; o->normal[1] = P[1]; o->normal[2] = P[2];
      if (++n >= maxc) return n;
    }
  }
  return n;
}

/* dCollideRayCylinder, ode/src/ray.cpp:500-698: the flat caps when the ray
 * starts inside the infinite cylinder and runs along the axis, else the curved
 * side between the caps. eps is dEpsilon of the build. */
static int collide_ray_cylinder(const GeomRef* ray, const GeomRef* cy, OContact* c) {
  const real* RR = ray->R;
  const real* CR = cy->R;
  const real half = cy->p[1] * 0.5;
  real r[3] = {ray->pos[0] - cy->pos[0], ray->pos[1] - cy->pos[1], ray->pos[2] - cy->pos[2]};
  real d = CR[2] * r[0] + CR[6] * r[1] + CR[10] * r[2];
  real q[3];
  for (int i = 0; i < 3; ++i) q[i] = (d * CR[i * 4 + 2]) - r[i];
  const real C = dot3(q, q) - (cy->p[0] * cy->p[0]);
  const real uv = CR[2] * RR[2] + CR[6] * RR[6] + CR[10] * RR[10];
  for (int i = 0; i < 3; ++i) r[i] = (uv * CR[i * 4 + 2]) - RR[i * 4 + 2];
  real A = dot3(r, r);
  const real B = 2 * dot3(q, r);
  real k = B * B - 4 * A * C;
  if (k < DBL_EPSILON && C <= 0) {
    const real uvsign = (uv < 0) ? -1.0 : 1.0;
    const real internal = (d >= -half && d <= +half) ? -1.0 : 1.0;
    if (((uv > 0) && (d + (uvsign * ray->p[0]) < half * internal)) ||
        ((uv < 0) && (d + (uvsign * ray->p[0]) > half * internal)))
      return 0;
    c->depth = ((-uvsign * d) - (internal * half));
    for (int i = 0; i < 3; ++i) {
      c->pos[i] = ray->pos[i] + (c->depth * RR[i * 4 + 2]);
      c->normal[i] = uvsign * (CR[i * 4 + 2]);
    }
    return 1;
  }
  if (k > 0) {
    k = sqrt(k);
    A = 1.0 / (2 * A);
    real alpha = (-B - k) * A;
    if (alpha < 0) alpha = (-B + k) * A;
    if (alpha >= 0 && alpha <= ray->p[0]) {
      for (int i = 0; i < 3; ++i) c->pos[i] = ray->pos[i] + (alpha * RR[i * 4 + 2]);
      for (int i = 0; i < 3; ++i) q[i] = c->pos[i] - cy->pos[i];
      d = q[0] * CR[2] + q[1] * CR[6] + q[2] * CR[10];
      if (d >= -half && d <= +half) {
        const real nsign = (C < 0) ? -1.0 : 1.0;
        for (int i = 0; i < 3; ++i) c->normal[i] = nsign * (c->pos[i] - (cy->pos[i] + d * CR[i * 4 + 2]));
        safe_normalize3(c->normal);
        c->depth = alpha;
        return 1;
      }
    }
  }
  return 0;
}

/* dCollideCylinderBox (ode/src/collision_cylinder_box.cpp:44-1036): separating
 * axes over the box faces, the cylinder axis, their cross products, the box
 * vertices and the box edges against both rims; then the cylinder's side edge
 * clipped by the box, or the box face clipped by the rim's octagon. */
typedef struct {
  real cR[12], cpos[3], caxis[3], crad, clen, cnorm[8][3];
  real bR[12], bpos[3], bhalf[3], bv[8][3];
  real diff[3], normal[3], best_depth, best_rb, best_rc;
  int best_axis;
} CylBox;

/* dMatrix3Inv, ode/src/collision_util.h:192-212, its operator precedence kept */
static void cb_mat3_inv(const real* ma, real* dst) {
  const real det = ma[0] * (ma[5] * ma[10] - ma[9] * ma[6]) - ma[1] * (ma[4] * ma[10] - ma[8] * ma[6]) +
                   ma[2] * (ma[4] * ma[9] - ma[8] * ma[5]);
  if (fabs(det) < 0.0005) {
    memset(dst, 0, 12 * sizeof(real));
    dst[0] = dst[5] = dst[10] = 1;
    return;
  }
  dst[0] = ma[5] * ma[10] - ma[6] * ma[9] / det;
  dst[1] = -(ma[1] * ma[10] - ma[9] * ma[2]) / det;
  dst[2] = ma[1] * ma[6] - ma[5] * ma[2] / det;
  dst[4] = -(ma[4] * ma[10] - ma[6] * ma[8]) / det;
  dst[5] = ma[0] * ma[10] - ma[8] * ma[2] / det;
  dst[6] = -(ma[0] * ma[6] - ma[4] * ma[2]) / det;
  dst[8] = ma[4] * ma[9] - ma[8] * ma[5] / det;
  dst[9] = -(ma[0] * ma[9] - ma[8] * ma[1]) / det;
  dst[10] = ma[0] * ma[5] - ma[1] * ma[4] / det;
  dst[3] = dst[7] = dst[11] = 0;
}

/* _cldTestAxis (collision_cylinder_box.cpp:206-285) */
static int cb_test_axis(CylBox* D, real* n, int iAxis) {
  const real fL = sqrt(dot3(n, n));
  if (fL < 1e-5) return 1;
  safe_normalize3(n);
  const real fdot1 = dot3(D->caxis, n);
  real frc;
  if (fdot1 > 1.0 || fdot1 < -1.0) frc = D->clen * 0.5;
  else frc = fabs(fdot1 * (D->clen * 0.5)) + D->crad * sqrt(1.0 - (fdot1 * fdot1));
  real frb = 0;
  for (int j = 0; j < 3; ++j) {
    const real col[3] = {D->bR[j], D->bR[4 + j], D->bR[8 + j]};
    frb += fabs(dot3(col, n)) * D->bhalf[j];
  }
  const real fd = dot3(D->diff, n);
  real fDepth = frc + frb;
  if (fabs(fd) > fDepth) return 0;
  fDepth -= fabs(fd);
  if (fDepth < D->best_depth) {
    D->best_depth = fDepth;
    D->normal[0] = n[0]; D->normal[1] = n[1]; D->normal[2] = n[2];
    D->best_axis = iAxis;
    D->best_rb = frb;
    D->best_rc = frc;
    if (fd > 0) { D->normal[0] = -D->normal[0]; D->normal[1] = -D->normal[1]; D->normal[2] = -D->normal[2]; }
  }
  return 1;
}

/* _cldTestEdgeCircleAxis (collision_cylinder_box.cpp:289-333) */
static int cb_test_edge_circle(CylBox* D, const real* cc, const real* v0, const real* v1, int iAxis) {
  real e[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
  safe_normalize3(e);
  const real fdot2 = dot3(e, D->caxis);
  if (fabs(fdot2) < 1e-5) return 1;
  real t1[3] = {cc[0] - v0[0], cc[1] - v0[1], cc[2] - v0[2]};
  const real fdot1 = dot3(t1, D->caxis);
  real p[3];
  for (int i = 0; i < 3; ++i) p[i] = v0[i] + e[i] * (fdot1 / fdot2);
  real tan_[3], ax[3];
  for (int i = 0; i < 3; ++i) t1[i] = cc[i] - p[i];
  cross3(tan_, t1, D->caxis);
  cross3(ax, tan_, e);
  return cb_test_axis(D, ax, iAxis);
}

/* dClipEdgeToPlane, ode/src/collision_util.cpp:471-510 */
static int cb_clip_edge(real* e0, real* e1, const real* pl) {
  const real d0 = pl[0] * e0[0] + pl[1] * e0[1] + pl[2] * e0[2] + pl[3];
  const real d1 = pl[0] * e1[0] + pl[1] * e1[1] + pl[2] * e1[2] + pl[3];
  if (d0 < 0 && d1 < 0) return 0;
  if (d0 > 0 && d1 > 0) return 1;
  if ((d0 > 0 && d1 < 0) || (d0 < 0 && d1 > 0)) {
    real ip[3];
    for (int i = 0; i < 3; ++i) ip[i] = e0[i] - (e0[i] - e1[i]) * d0 / (d0 - d1);
    real* dst = (d0 < 0) ? e0 : e1;
    dst[0] = ip[0]; dst[1] = ip[1]; dst[2] = ip[2];
  }
  return 1;
}

/* dClipPolyToPlane, ode/src/collision_util.cpp:512-553 */
#define CB_MAX_CLIP 16   /* MAX_CYLBOX_CLIP_POINTS; points beyond it are dropped */
static void cb_clip_poly(const real (*in)[3], int nin, real (*out)[3], int* nout, const real* pl) {
  int n = 0;
  for (int i1 = 0, i0 = nin - 1; i1 < nin; i0 = i1, i1++) {
    const real d0 = pl[0] * in[i0][0] + pl[1] * in[i0][1] + pl[2] * in[i0][2] + pl[3];
    const real d1 = pl[0] * in[i1][0] + pl[1] * in[i1][1] + pl[2] * in[i1][2] + pl[3];
    if (d0 >= 0 && n < CB_MAX_CLIP) { out[n][0] = in[i0][0]; out[n][1] = in[i0][1]; out[n][2] = in[i0][2]; n++; }
    if (((d0 > 0 && d1 < 0) || (d0 < 0 && d1 > 0)) && n < CB_MAX_CLIP) {
      for (int i = 0; i < 3; ++i) out[n][i] = in[i0][i] - (in[i0][i] - in[i1][i]) * d0 / (d0 - d1);
      n++;
    }
  }
  *nout = n;
}

static int collide_cylinder_box(const GeomRef* cy, const GeomRef* bx, unsigned flags, OContact* c) {
  const int maxc = (int)(flags & 0xffff);
  CylBox D;
  /* _cldInitCylinderBox, :100-203 */
  memcpy(D.cR, cy->R, sizeof(D.cR));
  for (int i = 0; i < 3; ++i) { D.cpos[i] = cy->pos[i]; D.caxis[i] = cy->R[i * 4 + 2]; }
  D.crad = cy->p[0];
  D.clen = cy->p[1];
  memcpy(D.bR, bx->R, sizeof(D.bR));
  for (int i = 0; i < 3; ++i) { D.bpos[i] = bx->pos[i]; D.bhalf[i] = bx->p[i] * 0.5; }
  static const signed char sgn[8][3] = {{-1, 1, -1}, {1, 1, -1}, {-1, -1, -1}, {1, -1, -1},
                                        {1, 1, 1},   {1, -1, 1}, {-1, -1, 1}, {-1, 1, 1}};
  for (int k = 0; k < 8; ++k) {
    const real v[3] = {sgn[k][0] * D.bhalf[0], sgn[k][1] * D.bhalf[1], sgn[k][2] * D.bhalf[2]};
    real w[3];
    mul0_331(w, D.bR, v);
    for (int i = 0; i < 3; ++i) D.bv[k][i] = w[i] + D.bpos[i];
  }
  for (int i = 0; i < 3; ++i) D.diff[i] = D.cpos[i] - D.bpos[i];
  {
    real ang = M_PI / 8;
    const real inc = ang * 2.0;
    for (int k = 0; k < 8; ++k) {
      D.cnorm[k][0] = -cos(ang);
      D.cnorm[k][1] = -sin(ang);
      D.cnorm[k][2] = 0;
      ang += inc;
    }
  }
  /* _cldTestSeparatingAxes, :336-574 */
  D.best_depth = INFINITY;
  D.best_axis = 0;
  D.best_rb = D.best_rc = 0;
  D.normal[0] = D.normal[1] = D.normal[2] = 0;
  real ax[3];
  for (int j = 0; j < 3; ++j) {
    ax[0] = D.bR[j]; ax[1] = D.bR[4 + j]; ax[2] = D.bR[8 + j];
    if (!cb_test_axis(&D, ax, 1 + j)) return 0;
  }
  ax[0] = D.caxis[0]; ax[1] = D.caxis[1]; ax[2] = D.caxis[2];
  if (!cb_test_axis(&D, ax, 4)) return 0;
  for (int j = 0; j < 3; ++j) {
    const real col[3] = {D.bR[j], D.bR[4 + j], D.bR[8 + j]};
    cross3(ax, D.caxis, col);
    if (dot3(ax, ax) > 1e-6 && !cb_test_axis(&D, ax, 5 + j)) return 0;
  }
  for (int k = 0; k < 8; ++k) {
    real t1[3] = {D.bv[k][0] - D.cpos[0], D.bv[k][1] - D.cpos[1], D.bv[k][2] - D.cpos[2]}, t2[3];
    cross3(t2, D.caxis, t1);
    cross3(ax, D.caxis, t2);
    if (dot3(ax, ax) > 1e-6 && !cb_test_axis(&D, ax, 8 + k)) return 0;
  }
  static const unsigned char edges[12][2] = {{1, 0}, {1, 3}, {2, 3}, {2, 0}, {4, 1}, {4, 7},
                                             {0, 7}, {5, 3}, {5, 6}, {2, 6}, {4, 5}, {6, 7}};
  for (int side = 0; side < 2; ++side) {   /* top rim, then bottom rim */
    real cc[3];
    for (int i = 0; i < 3; ++i) cc[i] = (side == 0) ? D.cpos[i] + D.caxis[i] * (D.clen * 0.5)
                                                     : D.cpos[i] - D.caxis[i] * (D.clen * 0.5);
    for (int e = 0; e < 12; ++e)
      if (!cb_test_edge_circle(&D, cc, D.bv[edges[e][0]], D.bv[edges[e][1]], 16 + 12 * side + e)) return 0;
  }
  if (D.best_axis == 0) return 0;
  int n = 0;
  const real fdot = dot3(D.normal, D.caxis);
  if (fabs(fdot) < 0.9) {
    /* _cldClipCylinderToBox, :576-717 */
    const real t = dot3(D.caxis, D.normal);
    real vN[3];
    for (int i = 0; i < 3; ++i) vN[i] = D.normal[i] - D.caxis[i] * t;
    safe_normalize3(vN);
    real e0[3], e1[3];
    for (int i = 0; i < 3; ++i) {
      const real ct = D.cpos[i] + vN[i] * D.crad;
      e0[i] = ct + D.caxis[i] * (D.clen * 0.5);
      e1[i] = ct - D.caxis[i] * (D.clen * 0.5);
    }
    for (int i = 0; i < 3; ++i) { e0[i] -= D.bpos[i]; e1[i] -= D.bpos[i]; }
    for (int sgn2 = 0; sgn2 < 2; ++sgn2)
      for (int j = 0; j < 3; ++j) {
        real pl[4] = {D.bR[j], D.bR[4 + j], D.bR[8 + j], D.bhalf[j]};
        if (sgn2) { pl[0] = -pl[0]; pl[1] = -pl[1]; pl[2] = -pl[2]; }
        if (!cb_clip_edge(e0, e1, pl)) return 0;
      }
    real d0 = D.best_rb + dot3(e0, D.normal);
    real d1 = D.best_rb + dot3(e1, D.normal);
    if (d0 < 0) d0 = 0;
    if (d1 < 0) d1 = 0;
    for (int i = 0; i < 3; ++i) { e0[i] += D.bpos[i]; e1[i] += D.bpos[i]; }
    c[n].depth = d0;
    for (int i = 0; i < 3; ++i) { c[n].normal[i] = -D.normal[i]; c[n].pos[i] = e0[i]; }
    n++;
    if (n != maxc) {
      c[n].depth = d1;
      for (int i = 0; i < 3; ++i) { c[n].normal[i] = -D.normal[i]; c[n].pos[i] = e1[i]; }
      n++;
    }
    return n;
  }
  /* _cldClipBoxToCylinder, :720-983 */
  real ccp[3], cn_rel[3] = {0, 0, 0};
  if (dot3(D.caxis, D.normal) > 0) {
    for (int i = 0; i < 3; ++i) ccp[i] = D.cpos[i] + D.caxis[i] * (D.clen * 0.5);
    cn_rel[2] = -1.0;
  } else {
    for (int i = 0; i < 3; ++i) ccp[i] = D.cpos[i] - D.caxis[i] * (D.clen * 0.5);
    cn_rel[2] = 1.0;
  }
  real binv[12], vNr[3];
  cb_mat3_inv(D.bR, binv);
  mul0_331(vNr, binv, D.normal);
  const real an[3] = {fabs(vNr[0]), fabs(vNr[1]), fabs(vNr[2])};
  int iB0, iB1, iB2;
  if (an[1] > an[0]) {
    if (an[0] > an[2]) { iB0 = 1; iB1 = 0; iB2 = 2; }
    else if (an[1] > an[2]) { iB0 = 1; iB1 = 2; iB2 = 0; }
    else { iB0 = 2; iB1 = 1; iB2 = 0; }
  } else {
    if (an[1] > an[2]) { iB0 = 0; iB1 = 1; iB2 = 2; }
    else if (an[0] > an[2]) { iB0 = 0; iB1 = 2; iB2 = 1; }
    else { iB0 = 2; iB1 = 0; iB2 = 1; }
  }
  real ctr[3];
  {
    const real col[3] = {D.bR[iB0], D.bR[4 + iB0], D.bR[8 + iB0]};
    for (int i = 0; i < 3; ++i)
      ctr[i] = (vNr[iB0] > 0) ? D.bpos[i] - D.bhalf[iB0] * col[i] : D.bpos[i] + D.bhalf[iB0] * col[i];
  }
  real pts[4][3], A1[16][3], A2[16][3];
  memset(A1, 0, sizeof(A1));
  memset(A2, 0, sizeof(A2));
  const real a1[3] = {D.bR[iB1], D.bR[4 + iB1], D.bR[8 + iB1]};
  const real a2[3] = {D.bR[iB2], D.bR[4 + iB2], D.bR[8 + iB2]};
  const real h1 = D.bhalf[iB1], h2 = D.bhalf[iB2];
  for (int i = 0; i < 3; ++i) {
    pts[0][i] = ctr[i] + h1 * a1[i] - h2 * a2[i];
    pts[1][i] = ctr[i] - h1 * a1[i] - h2 * a2[i];
    pts[2][i] = ctr[i] - h1 * a1[i] + h2 * a2[i];
    pts[3][i] = ctr[i] + h1 * a1[i] + h2 * a2[i];
  }
  real cinv[12];
  cb_mat3_inv(D.cR, cinv);
  for (int k = 0; k < 4; ++k) {
    const real t[3] = {pts[k][0] - ccp[0], pts[k][1] - ccp[1], pts[k][2] - ccp[2]};
    mul0_331(pts[k], cinv, t);
  }
  int n1 = 0, n2 = 0;
  real pl[4] = {cn_rel[0], cn_rel[1], cn_rel[2], 0.0};
  cb_clip_poly((const real(*)[3])pts, 4, A1, &n1, pl);
  int seg;
  for (seg = 0; seg < 8; ++seg) {
    pl[0] = D.cnorm[seg][0]; pl[1] = D.cnorm[seg][1]; pl[2] = D.cnorm[seg][2]; pl[3] = D.crad;
    if (seg % 2 == 0) cb_clip_poly((const real(*)[3])A1, n1, A2, &n2, pl);
    else cb_clip_poly((const real(*)[3])A2, n2, A1, &n1, pl);
  }
  const int np = (seg % 2) ? n2 : n1;
  real (*A)[3] = (seg % 2) ? A2 : A1;
  for (int k = 0; k < np; ++k) {
    real p[3];
    mul0_331(p, D.cR, A[k]);
    for (int i = 0; i < 3; ++i) p[i] += ccp[i];
    const real t[3] = {p[0] - D.cpos[0], p[1] - D.cpos[1], p[2] - D.cpos[2]};
    const real dep = D.best_rc - dot3(t, D.normal);
    if (dep > 0) {
      c[n].depth = dep;
      for (int i = 0; i < 3; ++i) { c[n].normal[i] = -D.normal[i]; c[n].pos[i] = p[i]; }
      if (++n == maxc) break;
    }
  }
  return n;
}

/* Collider table restricted to this path: returns the collider id for the
 * ordered class pair and whether the call is reversed, as dInitColliders
 * (ode/src/collision_kernel.cpp:167-268) arranges it. */
enum { C_NONE, C_SS, C_SB, C_SP, C_BB, C_BP, C_CP, C_HF, C_CS, C_CB, C_CC, C_RS, C_RB, C_RC, C_RP,
       C_YS, C_YB, C_YP, C_RY };
static int collider_of(int t1, int t2, int* reverse) {
  *reverse = 0;
#define PAIR(a, b, id) \
  if (t1 == (a) && t2 == (b)) return id; \
  if (t1 == (b) && t2 == (a)) { *reverse = ((a) != (b)); return id; }
  PAIR(ODEGPU_GEOM_SPHERE, ODEGPU_GEOM_SPHERE, C_SS);
  PAIR(ODEGPU_GEOM_SPHERE, ODEGPU_GEOM_BOX, C_SB);
  PAIR(ODEGPU_GEOM_SPHERE, ODEGPU_GEOM_PLANE, C_SP);
  PAIR(ODEGPU_GEOM_BOX, ODEGPU_GEOM_BOX, C_BB);
  PAIR(ODEGPU_GEOM_BOX, ODEGPU_GEOM_PLANE, C_BP);
  PAIR(ODEGPU_GEOM_CAPSULE, ODEGPU_GEOM_SPHERE, C_CS);
  PAIR(ODEGPU_GEOM_CAPSULE, ODEGPU_GEOM_BOX, C_CB);
  PAIR(ODEGPU_GEOM_CAPSULE, ODEGPU_GEOM_CAPSULE, C_CC);
  PAIR(ODEGPU_GEOM_CAPSULE, ODEGPU_GEOM_PLANE, C_CP);
  PAIR(ODEGPU_GEOM_HEIGHTFIELD, ODEGPU_GEOM_SPHERE, C_HF);
  PAIR(ODEGPU_GEOM_HEIGHTFIELD, ODEGPU_GEOM_BOX, C_HF);
  PAIR(ODEGPU_GEOM_HEIGHTFIELD, ODEGPU_GEOM_CAPSULE, C_HF);
  PAIR(ODEGPU_GEOM_RAY, ODEGPU_GEOM_SPHERE, C_RS);
  PAIR(ODEGPU_GEOM_RAY, ODEGPU_GEOM_BOX, C_RB);
  PAIR(ODEGPU_GEOM_RAY, ODEGPU_GEOM_CAPSULE, C_RC);
  PAIR(ODEGPU_GEOM_RAY, ODEGPU_GEOM_PLANE, C_RP);
  PAIR(ODEGPU_GEOM_HEIGHTFIELD, ODEGPU_GEOM_RAY, C_HF);
  /* cylinder-cylinder and capsule-cylinder need libccd (collision_kernel.cpp:215-220) */
  PAIR(ODEGPU_GEOM_CYLINDER, ODEGPU_GEOM_SPHERE, C_YS);
  PAIR(ODEGPU_GEOM_CYLINDER, ODEGPU_GEOM_BOX, C_YB);
  PAIR(ODEGPU_GEOM_CYLINDER, ODEGPU_GEOM_PLANE, C_YP);
  PAIR(ODEGPU_GEOM_RAY, ODEGPU_GEOM_CYLINDER, C_RY);
  PAIR(ODEGPU_GEOM_HEIGHTFIELD, ODEGPU_GEOM_CYLINDER, C_HF);
#undef PAIR
  return C_NONE;
}

int oracle_heightfield_collide(const GeomRef* hf, const GeomRef* o2, unsigned flags, OContact* c);

/* dCollide, ode/src/collision_kernel.cpp:292-340: dispatch, reversing the
 * call and negating normals for reversed class pairs. */
static int do_collide(const GeomRef* g1, const GeomRef* g2, unsigned flags, OContact* c) {
  if ((flags & 0xffff) == 0) return 0;
  int rev;
  int id = collider_of(g1->type, g2->type, &rev);
  const GeomRef* a = rev ? g2 : g1;
  const GeomRef* b = rev ? g1 : g2;
  int n = 0;
  switch (id) {
    case C_SS: n = collide_spheres(a->pos, a->p[0], b->pos, b->p[0], c); break;
    case C_SB: n = collide_sphere_box(a, b, c); break;
    case C_SP: n = collide_sphere_plane(a, b, c); break;
    case C_BB: n = collide_box_box(a, b, flags, c); break;
    case C_BP: n = collide_box_plane(a, b, flags, c); break;
    case C_CP: n = collide_capsule_plane(a, b, flags, c); break;
    case C_CS: n = collide_capsule_sphere(a, b, c); break;
    case C_CB: n = collide_capsule_box(a, b, c); break;
    case C_CC: n = collide_capsule_capsule(a, b, flags, c); break;
    case C_HF: n = oracle_heightfield_collide(a, b, flags, c); break;
    case C_RS: n = collide_ray_sphere(a, b, c); break;
    case C_RB: n = collide_ray_box(a, b, c); break;
    case C_RC: n = collide_ray_capsule(a, b, c); break;
    case C_RP: n = collide_ray_plane(a, b, c); break;
    case C_YS: n = collide_cylinder_sphere(a, b, c); break;
    case C_YB: n = collide_cylinder_box(a, b, flags, c); break;
    case C_YP: n = collide_cylinder_plane(a, b, flags, c); break;
    case C_RY: n = collide_ray_cylinder(a, b, c); break;
    default: n = 0;
  }
  if (rev) {
    for (int i = 0; i < n; ++i) {
      c[i].normal[0] = -c[i].normal[0]; c[i].normal[1] = -c[i].normal[1]; c[i].normal[2] = -c[i].normal[2];
    }
  }
  return n;
}

/* ---- heightfield (ode/src/heightfield.cpp, dDOUBLE build: dEpsilon = DBL_EPSILON) ---- */

#define HF_EPS DBL_EPSILON
#define HF_MAXC_PER_CELL 10   /* HEIGHTFIELDMAXCONTACTPERCELL, ode/src/heightfield.h:14 */

typedef struct {
  const odegpuHeightfield* H;
  real sw, sd, inv_sw, inv_sd, zx_aspect, half_w, half_d;
} HFData;

/* dxHeightfieldData::SetData caches, heightfield.cpp:107-143 */
static void hf_data(const odegpuHeightfield* H, HFData* D) {
  D->H = H;
  D->half_w = H->width / 2.0;
  D->half_d = H->depth / 2.0;
  D->sw = H->width / (H->nx - 1.0);
  D->sd = H->depth / (H->nz - 1.0);
  D->zx_aspect = D->sd / D->sw;
  D->inv_sw = 1.0 / D->sw;
  D->inv_sd = 1.0 / D->sd;
}

/* GetHeight(int, int), heightfield.cpp:302-364 (double samples) */
static real hf_height(const HFData* D, int x, int z) {
  const odegpuHeightfield* H = D->H;
  if (H->wrap == 0) {
    if (x < 0) x = 0;
    if (z < 0) z = 0;
    if (x > H->nx - 1) x = H->nx - 1;
    if (z > H->nz - 1) z = H->nz - 1;
  } else {
    x %= H->nx - 1;
    z %= H->nz - 1;
    if (x < 0) x += H->nx - 1;
    if (z < 0) z += H->nz - 1;
  }
  const real h = H->heights[x + z * H->nx];
  return h * H->scale + H->offset;
}

/* IsOnHeightfield2, heightfield.cpp:241-299: is pos over the up (ABC, corner
 * A) or down (DBC, corner D) triangle of a cell */
static int hf_on_triangle(const HFData* D, const real* corner, const int* coords, const real* pos, int up) {
  if (up) {
    const real minx = corner[0];
    if (pos[0] < minx) return 0;
    const real maxx = (coords[0] + 1) * D->sw;
    if (pos[0] >= maxx) return 0;
    const real minz = corner[2];
    if (pos[2] < minz) return 0;
    const real maxz = (coords[1] + 1) * D->sd;
    if (pos[2] >= maxz) return 0;
    return (maxz - pos[2]) > (pos[0] - minx) * D->zx_aspect;
  } else {
    const real maxx = corner[0];
    if (pos[0] >= maxx) return 0;
    const real minx = (coords[0] - 1) * D->sw;
    if (pos[0] < minx) return 0;
    const real maxz = corner[2];
    if (pos[2] >= maxz) return 0;
    const real minz = (coords[1] - 1) * D->sd;
    if (pos[2] < minz) return 0;
    return (maxz - pos[2]) <= (pos[0] - minx) * D->zx_aspect;
  }
}

/* computeAABB of sphere / box / capsule / ray (sphere.cpp:59-67,
 * box.cpp:60-78, capsule.cpp:60-74, ray.cpp:56-89) */
static void geom_aabb(const GeomRef* g, real* aabb) {
  const real* R = g->R;
  const real* pos = g->pos;
  real xr, yr, zr;
  if (g->type == ODEGPU_GEOM_RAY) {
    for (int i = 0; i < 3; ++i) {
      const real e = pos[i] + R[i * 4 + 2] * g->p[0];
      aabb[2 * i] = pos[i] < e ? pos[i] : e;
      aabb[2 * i + 1] = pos[i] < e ? e : pos[i];
    }
    return;
  }
  if (g->type == ODEGPU_GEOM_SPHERE) {
    xr = yr = zr = g->p[0];
  } else if (g->type == ODEGPU_GEOM_CYLINDER) {   /* cylinder.cpp:58-73 */
    const real radius = g->p[0], lz = g->p[1];
    xr = fabs(R[0] * radius) + fabs(R[1] * radius) + 0.5 * fabs(R[2] * lz);
    yr = fabs(R[4] * radius) + fabs(R[5] * radius) + 0.5 * fabs(R[6] * lz);
    zr = fabs(R[8] * radius) + fabs(R[9] * radius) + 0.5 * fabs(R[10] * lz);
  } else if (g->type == ODEGPU_GEOM_BOX) {
    const real* side = g->p;
    xr = 0.5 * (fabs(R[0] * side[0]) + fabs(R[1] * side[1]) + fabs(R[2] * side[2]));
    yr = 0.5 * (fabs(R[4] * side[0]) + fabs(R[5] * side[1]) + fabs(R[6] * side[2]));
    zr = 0.5 * (fabs(R[8] * side[0]) + fabs(R[9] * side[1]) + fabs(R[10] * side[2]));
  } else {
    const real radius = g->p[0], lz = g->p[1];
    xr = fabs(R[2] * lz) * 0.5 + radius;
    yr = fabs(R[6] * lz) * 0.5 + radius;
    zr = fabs(R[10] * lz) * 0.5 + radius;
  }
  aabb[0] = pos[0] - xr; aabb[1] = pos[0] + xr;
  aabb[2] = pos[1] - yr; aabb[3] = pos[1] + yr;
  aabb[4] = pos[2] - zr; aabb[5] = pos[2] + zr;
}

/* dGeomSpherePointDepth (sphere.cpp:95-105), dGeomBoxPointDepth
 * (box.cpp:109-172), dGeomCapsulePointDepth (capsule.cpp:104-126) */
static real geom_point_depth(const GeomRef* g, const real* v) {
  const real* pos = g->pos;
  const real* R = g->R;
  if (g->type == ODEGPU_GEOM_SPHERE) {
    return g->p[0] - sqrt((v[0] - pos[0]) * (v[0] - pos[0]) + (v[1] - pos[1]) * (v[1] - pos[1]) +
                          (v[2] - pos[2]) * (v[2] - pos[2]));
  }
  if (g->type == ODEGPU_GEOM_BOX) {
    real p[3] = {v[0] - pos[0], v[1] - pos[1], v[2] - pos[2]}, q[3], dist[6];
    mul1_331(q, R, p);
    int inside = 1;
    for (int i = 0; i < 3; i++) {
      const real side = g->p[i] * 0.5;
      dist[i] = side - q[i];
      dist[i + 3] = side + q[i];
      if ((dist[i] < 0) || (dist[i + 3] < 0)) inside = 0;
    }
    if (inside) {
      real smallest = (real)(unsigned)-1;
      for (int i = 0; i < 6; i++)
        if (dist[i] < smallest) smallest = dist[i];
      return smallest;
    }
    real largest = 0;
    for (int i = 0; i < 6; i++)
      if (dist[i] > largest) largest = dist[i];
    return -largest;
  }
  real a[3] = {v[0] - pos[0], v[1] - pos[1], v[2] - pos[2]};
  real beta = a[0] * R[2] + a[1] * R[6] + a[2] * R[10];
  const real lz2 = g->p[1] * 0.5;
  if (beta < -lz2) beta = -lz2;
  else if (beta > lz2) beta = lz2;
  a[0] = pos[0] + beta * R[2];
  a[1] = pos[1] + beta * R[6];
  a[2] = pos[2] + beta * R[10];
  return g->p[0] - sqrt((v[0] - a[0]) * (v[0] - a[0]) + (v[1] - a[1]) * (v[1] - a[1]) +
                        (v[2] - a[2]) * (v[2] - a[2]));
}

static int geom_plane_collide(const GeomRef* g, const GeomRef* pl, unsigned flags, OContact* c) {
  switch (g->type) {
    case ODEGPU_GEOM_SPHERE: return collide_sphere_plane(g, pl, c);
    case ODEGPU_GEOM_BOX: return collide_box_plane(g, pl, flags, c);
    case ODEGPU_GEOM_RAY: return collide_ray_plane(g, pl, c);
    case ODEGPU_GEOM_CYLINDER: return collide_cylinder_plane(g, pl, flags, c);
    default: return collide_capsule_plane(g, pl, flags, c);
  }
}

typedef struct {
  real v[3];
  int coords[2];
  int state;
} HFVertex;

typedef struct {
  int vi[3];          /* indices into the zone's vertex array */
  real plane[4];
  real maxy;
  int up, state;
} HFTri;

typedef struct {
  real plane[4];
  real maxy;
  int first, count;   /* triangles of the plane in the member list */
} HFPlane;

/* dxHeightfield::dCollideHeightfieldZone, heightfield.cpp:952-1676 (the edge
 * pass is compiled out in the reference). o2 is in heightfield space. */
static int hf_zone(const HFData* D, int minX, int maxX, int minZ, int maxZ, const GeomRef* o2,
                   const real* aabb, int max_contacts, unsigned flags, OContact* out) {
  const int numX = (maxX - minX) + 1, numZ = (maxZ - minZ) + 1;
  const real minO2 = aabb[2], maxO2 = aabb[3];
  HFVertex* V = (HFVertex*)calloc((size_t)numX * numZ, sizeof(HFVertex));
  real maxY = -INFINITY, minY = INFINITY;
  for (int xl = 0, x = minX; xl < numX; ++x, ++xl) {
    const real xpos = x * D->sw;
    for (int zl = 0, z = minZ; zl < numZ; ++z, ++zl) {
      const real zpos = z * D->sd;
      const real h = hf_height(D, x, z);
      HFVertex* hv = &V[xl * numZ + zl];
      hv->v[0] = xpos; hv->v[1] = h; hv->v[2] = zpos;
      hv->coords[0] = x; hv->coords[1] = z;
      maxY = fmax(maxY, h);
      minY = fmin(minY, h);
    }
  }
  if (minO2 - maxY > -HF_EPS) { free(V); return 0; }      /* totally above */
  if (minY - maxO2 > -HF_EPS) {                            /* totally under */
    out[0].pos[0] = o2->pos[0]; out[0].pos[1] = minY; out[0].pos[2] = o2->pos[2];
    out[0].normal[0] = 0; out[0].normal[1] = -1; out[0].normal[2] = 0;
    out[0].depth = minY - maxO2;
    free(V);
    return 1;
  }
  int nc = 0;
  int further = 0;
  if (o2->type != ODEGPU_GEOM_RAY) {   /* rays take the plane pass only */
    const real xratio = (aabb[1] - aabb[0]) * D->inv_sw;
    if (xratio > 1.5) further = 1;
    else {
      const real zratio = (aabb[5] - aabb[4]) * D->inv_sd;
      if (zratio > 1.5) further = 1;
    }
  }
  const int maxXl = maxX - minX, maxZl = maxZ - minZ;
  HFTri* T = (HFTri*)calloc((size_t)2 * (maxXl > 0 ? maxXl : 1) * (maxZl > 0 ? maxZl : 1), sizeof(HFTri));
  int numTri = 0;
  for (int xl = 0; xl < maxXl; ++xl) {
    int ic = xl * numZ, id = (xl + 1) * numZ;       /* C, D of z_local 0 */
    for (int zl = 0; zl < maxZl; ++zl) {
      const int ia = ic, ib = id;
      ic = xl * numZ + zl + 1;
      id = (xl + 1) * numZ + zl + 1;
      const real ah = V[ia].v[1], bh = V[ib].v[1], ch = V[ic].v[1], dh = V[id].v[1];
      const int ac = ah > minO2, bc = bh > minO2, cc = ch > minO2, dc = dh > minO2;
      V[ia].state = !ac; V[ib].state = !bc; V[ic].state = !cc; V[id].state = !dc;
      if (ac || bc || cc) {
        HFTri* t = &T[numTri++];
        t->state = 0;
        t->vi[0] = ia; t->vi[1] = ib; t->vi[2] = ic;
        t->maxy = ah > bh ? ah : bh;
        t->maxy = ch > t->maxy ? ch : t->maxy;
        t->up = 1;
      }
      if (bc || cc || dc) {
        HFTri* t = &T[numTri++];
        t->state = 0;
        t->vi[0] = id; t->vi[1] = ib; t->vi[2] = ic;
        t->maxy = dh > bh ? dh : bh;
        t->maxy = ch > t->maxy ? ch : t->maxy;
        t->up = 0;
      }
      if (further && (bc || cc) && (ah > ch && ah > bh && dh > ch && dh > bh)) {
        V[ib].state = 1;    /* concave edge BC */
        V[ic].state = 1;
      }
    }
  }
  /* pass 1: triangle planes, grouped by plane, sorted by height */
  for (int k = 0; k < numTri; ++k) {
    HFTri* t = &T[k];
    const real* v0 = V[t->vi[0]].v;
    const real* v1 = V[t->vi[1]].v;
    const real* v2 = V[t->vi[2]].v;
    real e1[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
    real e2[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
    real n[3];
    if (t->up) cross3(n, e1, e2);
    else cross3(n, e2, e1);
    const real il = 1.0 / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] *= il; n[1] *= il; n[2] *= il;
    t->plane[0] = n[0]; t->plane[1] = n[1]; t->plane[2] = n[2];
    t->plane[3] = dot3(n, v0);
  }
  HFPlane* P = (HFPlane*)calloc(numTri > 0 ? numTri : 1, sizeof(HFPlane));
  int* members = (int*)calloc(numTri > 0 ? numTri : 1, sizeof(int));
  int numPlanes = 0, nmem = 0;
  for (int k = 0; k < numTri; ++k) {
    HFTri* tb = &T[k];
    if (tb->state) continue;
    HFPlane* pl = &P[numPlanes];
    pl->first = nmem;
    pl->count = 0;
    members[nmem++] = k; pl->count++;
    for (int q = 0; q < 4; ++q) pl->plane[q] = tb->plane[q];
    for (int m = k + 1; m < numTri; ++m) {
      HFTri* tt = &T[m];
      if (tt->state) continue;
      if (fabs(tb->plane[1] - tt->plane[1]) < HF_EPS && fabs(tb->plane[3] - tt->plane[3]) < HF_EPS &&
          fabs(tb->plane[0] - tt->plane[0]) < HF_EPS && fabs(tb->plane[2] - tt->plane[2]) < HF_EPS) {
        members[nmem++] = m; pl->count++;
        tt->state = 1;
      }
    }
    tb->state = 1;
    pl->maxy = T[members[pl->first]].maxy;
    for (int q = 1; q < pl->count; ++q)
      if (T[members[pl->first + q]].maxy > pl->maxy) pl->maxy = T[members[pl->first + q]].maxy;
    numPlanes++;
  }
  /* sortPlanes (heightfield.cpp:910-932): bubble sort, descending height */
  {
    int swapped = 1;
    while (swapped) {
      swapped = 0;
      for (int i = 0; i < numPlanes - 1; ++i) {
        if ((P[i].maxy - P[i + 1].maxy) > HF_EPS) {
          HFPlane tmp = P[i]; P[i] = P[i + 1]; P[i + 1] = tmp;
          swapped = 1;
        }
      }
    }
  }
  const unsigned plane_flags = (flags & ~0xffffu) | HF_MAXC_PER_CELL;
  for (int k = 0; k < numPlanes; ++k) {
    HFPlane* pl = &P[k];
    GeomRef gp;
    memset(&gp, 0, sizeof(gp));
    gp.type = ODEGPU_GEOM_PLANE;
    gp.p = pl->plane;
    OContact pc[HF_MAXC_PER_CELL];
    int did = 0;
    const int npc = geom_plane_collide(o2, &gp, plane_flags, pc);
    for (int i = 0; i < npc; ++i) {
      for (int b = 0; b < pl->count; ++b) {
        const HFTri* t = &T[members[pl->first + b]];
        const HFVertex* cv = &V[t->vi[0]];
        if (hf_on_triangle(D, cv->v, cv->coords, pc[i].pos, t->up)) {
          OContact* o = &out[nc];
          for (int q = 0; q < 3; ++q) { o->pos[q] = pc[i].pos[q]; o->normal[q] = -pl->plane[q]; }
          o->depth = pc[i].depth;
          nc++;
          if (nc == max_contacts) goto done;
          did = 1;
          break;
        }
      }
    }
    if (did) {
      for (int b = 0; b < pl->count; ++b) {
        const HFTri* t = &T[members[pl->first + b]];
        for (int i = 0; i < 3; ++i) V[t->vi[i]].state = 1;
      }
    } else {
      for (int b = 0; b < pl->count; ++b) T[members[pl->first + b]].state = 0;
    }
  }
  /* pass 2: triangle vertices against the geom's point depth */
  if (further) {
    for (int k = 0; k < numTri; ++k) {
      const HFTri* t = &T[k];
      if (t->state) continue;
      for (int i = 0; i < 3; ++i) {
        HFVertex* hv = &V[t->vi[i]];
        if (hv->state) continue;
        real depth;
        int hit;
        if (o2->type == ODEGPU_GEOM_CYLINDER) {
          /* no point-depth function for cylinders: a ray from the vertex along
           * the triangle's normal, of length (minO2 - y) * 1000, and the ray's
           * depth (heightfield.cpp:1562-1584) */
          real rR[12] = {1, 0, t->plane[0], 0, 0, 1, t->plane[1], 0, 0, 0, t->plane[2], 0};
          real rp[4] = {(minO2 - hv->v[1]) * 1000.0, 0, 0, 0};
          GeomRef ray = {ODEGPU_GEOM_RAY, hv->v, rR, rp, NULL};
          OContact rc;
          hit = collide_ray_cylinder(&ray, o2, &rc);
          depth = rc.depth;
        } else {
          depth = geom_point_depth(o2, hv->v);
          hit = depth > HF_EPS;
        }
        if (hit) {
          OContact* o = &out[nc];
          for (int q = 0; q < 3; ++q) { o->pos[q] = hv->v[q]; o->normal[q] = -t->plane[q]; }
          o->depth = depth;
          nc++;
          if (nc == max_contacts) goto done;
          hv->state = 1;
        }
      }
    }
  }
done:
  free(V); free(T); free(P); free(members);
  return nc;
}

/* dCollideHeightfield, heightfield.cpp:1677-1853 (placeable heightfield,
 * centred origin: DHEIGHTFIELD_CORNER_ORIGIN undefined). */
int oracle_heightfield_collide(const GeomRef* hf, const GeomRef* o2, unsigned flags, OContact* c) {
  const int maxc = (int)(flags & 0xffff);
  if (maxc < 1 || !hf->g || !hf->g->hf) return 0;
  HFData D;
  hf_data(hf->g->hf, &D);
  const odegpuHeightfield* H = hf->g->hf;
  /* o2 into heightfield space */
  real p0[3] = {o2->pos[0] - hf->pos[0], o2->pos[1] - hf->pos[1], o2->pos[2] - hf->pos[2]};
  real pos1[3], R1[12];
  mul1_331(pos1, hf->R, p0);
  /* dMultiply1_333(R1, Rhf, Ro2) = Rhf^T Ro2 */
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j)
      R1[i * 4 + j] = hf->R[0 * 4 + i] * o2->R[0 * 4 + j] + hf->R[1 * 4 + i] * o2->R[1 * 4 + j] +
                      hf->R[2 * 4 + i] * o2->R[2 * 4 + j];
    R1[i * 4 + 3] = 0;
  }
  pos1[0] += D.half_w;
  pos1[2] += D.half_d;
  GeomRef g2 = *o2;
  g2.pos = pos1;
  g2.R = R1;
  real aabb[6];
  geom_aabb(&g2, aabb);
  const int wrapped = H->wrap != 0;
  if (!wrapped) {
    if (aabb[0] > H->width || aabb[4] > H->depth) return 0;
    if (aabb[1] < 0 || aabb[5] < 0) return 0;
  }
  int nMinX = (int)floor(nextafter(aabb[0] * D.inv_sw, -INFINITY));
  int nMaxX = (int)ceil(nextafter(aabb[1] * D.inv_sw, INFINITY));
  int nMinZ = (int)floor(nextafter(aabb[4] * D.inv_sd, -INFINITY));
  int nMaxZ = (int)ceil(nextafter(aabb[5] * D.inv_sd, INFINITY));
  if (!wrapped) {
    nMinX = nMinX > 0 ? nMinX : 0;
    nMaxX = nMaxX < H->nx - 1 ? nMaxX : H->nx - 1;
    nMinZ = nMinZ > 0 ? nMinZ : 0;
    nMaxZ = nMaxZ < H->nz - 1 ? nMaxZ : H->nz - 1;
  }
  const int n = hf_zone(&D, nMinX, nMaxX, nMinZ, nMaxZ, &g2, aabb, maxc, flags, c);
  /* contacts back to world space */
  for (int i = 0; i < n; ++i) {
    real q[3] = {c[i].pos[0] - D.half_w, c[i].pos[1], c[i].pos[2] - D.half_d};
    real w[3];
    mul0_331(w, hf->R, q);
    for (int k = 0; k < 3; ++k) c[i].pos[k] = w[k] + hf->pos[k];
    real nn[3] = {c[i].normal[0], c[i].normal[1], c[i].normal[2]};
    mul0_331(c[i].normal, hf->R, nn);
  }
  return n;
}

static void fill_ref(const OWorld* W, int gi, GeomRef* r) {
  const OGeom* g = &W->geom[gi];
  r->type = g->type;
  r->p = g->p;
  r->g = g;
  if (g->body >= 0) {
    r->pos = W->body[g->body].pos;
    r->R = W->body[g->body].R;
  } else {
    r->pos = g->hpos;
    r->R = g->hR;
  }
}

/* ------------------------------------------------------------------------ */
/* joints: getInfo1 / getInfo2                                              */

typedef struct {
  real fps, erp;
  real *J1l, *J1a, *J2l, *J2a;
  int rowskip;
  real *c, *cfm, *lo, *hi;
  int* findex;
} Info2;

/* setBall, ode/src/joints/joint.cpp:85-128 */
static void set_ball(OWorld* W, OJoint* J, Info2* info, const real* anchor1, const real* anchor2) {
  real a1[3], a2[3];
  int s = info->rowskip;
  OBody* B1 = &W->body[J->b[0]];
  info->J1l[0] = 1; info->J1l[s + 1] = 1; info->J1l[2 * s + 2] = 1;
  mul0_331(a1, B1->R, anchor1);
  /* dSetCrossMatrixMinus(J1a, a1, s) */
  info->J1a[1] = +a1[2]; info->J1a[2] = -a1[1];
  info->J1a[s + 0] = -a1[2]; info->J1a[s + 2] = +a1[0];
  info->J1a[2 * s + 0] = +a1[1]; info->J1a[2 * s + 1] = -a1[0];
  if (J->b[1] >= 0) {
    OBody* B2 = &W->body[J->b[1]];
    info->J2l[0] = -1; info->J2l[s + 1] = -1; info->J2l[2 * s + 2] = -1;
    mul0_331(a2, B2->R, anchor2);
    /* dSetCrossMatrixPlus(J2a, a2, s) */
    info->J2a[1] = -a2[2]; info->J2a[2] = +a2[1];
    info->J2a[s + 0] = +a2[2]; info->J2a[s + 2] = -a2[0];
    info->J2a[2 * s + 0] = -a2[1]; info->J2a[2 * s + 1] = +a2[0];
  }
  real k = info->fps * info->erp;
  if (J->b[1] >= 0) {
    OBody* B2 = &W->body[J->b[1]];
    for (int j = 0; j < 3; j++) info->c[j] = k * (a2[j] + B2->pos[j] - a1[j] - B1->pos[j]);
  } else {
    for (int j = 0; j < 3; j++) info->c[j] = k * (anchor2[j] - a1[j] - B1->pos[j]);
  }
}

/* setBall2, ode/src/joints/joint.cpp:134-196 */
static void set_ball2(OWorld* W, OJoint* J, Info2* info, const real* anchor1, const real* anchor2,
                      const real* axis, real erp1) {
  real a1[3], a2[3], q1[3], q2[3];
  int i, s = info->rowskip;
  OBody* B1 = &W->body[J->b[0]];
  plane_space(axis, q1, q2);
  for (i = 0; i < 3; i++) info->J1l[i] = axis[i];
  for (i = 0; i < 3; i++) info->J1l[s + i] = q1[i];
  for (i = 0; i < 3; i++) info->J1l[2 * s + i] = q2[i];
  mul0_331(a1, B1->R, anchor1);
  cross3(info->J1a, a1, axis);
  cross3(info->J1a + s, a1, q1);
  cross3(info->J1a + 2 * s, a1, q2);
  if (J->b[1] >= 0) {
    OBody* B2 = &W->body[J->b[1]];
    for (i = 0; i < 3; i++) info->J2l[i] = -axis[i];
    for (i = 0; i < 3; i++) info->J2l[s + i] = -q1[i];
    for (i = 0; i < 3; i++) info->J2l[2 * s + i] = -q2[i];
    mul0_331(a2, B2->R, anchor2);
    real* J2a = info->J2a;
    cross3(J2a, a2, axis); J2a[0] = -J2a[0]; J2a[1] = -J2a[1]; J2a[2] = -J2a[2];
    cross3(J2a + s, a2, q1); J2a[s] = -J2a[s]; J2a[s + 1] = -J2a[s + 1]; J2a[s + 2] = -J2a[s + 2];
    cross3(J2a + 2 * s, a2, q2);
    J2a[2 * s] = -J2a[2 * s]; J2a[2 * s + 1] = -J2a[2 * s + 1]; J2a[2 * s + 2] = -J2a[2 * s + 2];
  }
  real k1 = info->fps * erp1;
  real k = info->fps * info->erp;
  for (i = 0; i < 3; i++) a1[i] += B1->pos[i];
  real d[3];
  if (J->b[1] >= 0) {
    OBody* B2 = &W->body[J->b[1]];
    for (i = 0; i < 3; i++) a2[i] += B2->pos[i];
    d[0] = a2[0] - a1[0]; d[1] = a2[1] - a1[1]; d[2] = a2[2] - a1[2];
  } else {
    d[0] = anchor2[0] - a1[0]; d[1] = anchor2[1] - a1[1]; d[2] = anchor2[2] - a1[2];
  }
  info->c[0] = k1 * dot3(axis, d);
  info->c[1] = k * dot3(q1, d);
  info->c[2] = k * dot3(q2, d);
}

/* getHingeAngleFromRelativeQuat, ode/src/joints/joint.cpp:381-420 */
static real hinge_angle_from_qrel(const real* qrel, const real* axis) {
  real cost2 = qrel[0];
  real sint2 = sqrt(qrel[1] * qrel[1] + qrel[2] * qrel[2] + qrel[3] * qrel[3]);
  real theta = (dot3(qrel + 1, axis) >= 0) ? (2 * atan2(sint2, cost2)) : (2 * atan2(sint2, -cost2));
  if (theta > R_PI) theta -= (real)(2 * R_PI);
  theta = -theta;
  return theta;
}
/* getHingeAngle, ode/src/joints/joint.cpp:432-450 */
static real hinge_angle(OWorld* W, OJoint* J) {
  real qrel[4];
  const real* q1 = W->body[J->b[0]].q;
  if (J->b[1] >= 0) {
    real qq[4];
    qmul1(qq, q1, W->body[J->b[1]].q);
    qmul2(qrel, qq, J->qrel);
  } else {
    qmul3(qrel, q1, J->qrel);
  }
  return hinge_angle_from_qrel(qrel, J->axis1);
}

/* dxJointLimitMotor::testRotationalLimit, ode/src/joints/joint.cpp:534-553 */
static int limot_test(OLimot* L, real angle) {
  if (angle <= L->lostop) { L->limit = 1; L->limit_err = angle - L->lostop; return 1; }
  if (angle >= L->histop) { L->limit = 2; L->limit_err = angle - L->histop; return 1; }
  L->limit = 0;
  return 0;
}

/* dxJointLimitMotor::addLimot, ode/src/joints/joint.cpp:556-733. A linear
 * limot (rotational = 0, the slider's) works on J1l/J2l and, between two
 * bodies, puts the torque-decoupling vector ltd = (x2 - x1)/2 x ax1 in both
 * angular parts. */
static int limot_add(OWorld* W, OJoint* J, OLimot* L, Info2* info, int row, const real* ax1, int rotational) {
  int srow = row * info->rowskip;
  int powered = L->fmax > 0;
  if (!(powered || L->limit)) return 0;
  real* J1 = rotational ? info->J1a : info->J1l;
  real* J2 = rotational ? info->J2a : info->J2l;
  J1[srow + 0] = ax1[0]; J1[srow + 1] = ax1[1]; J1[srow + 2] = ax1[2];
  if (J->b[1] >= 0) { J2[srow + 0] = -ax1[0]; J2[srow + 1] = -ax1[1]; J2[srow + 2] = -ax1[2]; }
  real ltd[3] = {0, 0, 0};
  if (!rotational && J->b[1] >= 0) {
    const real* p1 = W->body[J->b[0]].pos;
    const real* p2 = W->body[J->b[1]].pos;
    real c[3] = {0.5 * (p2[0] - p1[0]), 0.5 * (p2[1] - p1[1]), 0.5 * (p2[2] - p1[2])};
    cross3(ltd, c, ax1);
    for (int k = 0; k < 3; ++k) { info->J1a[srow + k] = ltd[k]; info->J2a[srow + k] = ltd[k]; }
  }
  if (L->limit && (L->lostop == L->histop)) powered = 0;
  if (powered) {
    info->cfm[row] = L->normal_cfm;
    if (!L->limit) {
      info->c[row] = L->vel;
      info->lo[row] = -L->fmax;
      info->hi[row] = L->fmax;
    } else {
      real fm = L->fmax;
      if ((L->vel > 0) || (L->vel == 0 && L->limit == 2)) fm = -fm;
      if ((L->limit == 1 && L->vel > 0) || (L->limit == 2 && L->vel < 0)) fm *= L->fudge;
      OBody* B1 = &W->body[J->b[0]];
      OBody* B2 = J->b[1] >= 0 ? &W->body[J->b[1]] : 0;
      if (rotational) {
        for (int k = 0; k < 3; ++k) B1->tacc[k] += -fm * ax1[k];
        if (B2) for (int k = 0; k < 3; ++k) B2->tacc[k] += fm * ax1[k];
      } else {
        for (int k = 0; k < 3; ++k) B1->facc[k] += -fm * ax1[k];
        if (B2) {
          for (int k = 0; k < 3; ++k) B2->facc[k] += fm * ax1[k];
          for (int k = 0; k < 3; ++k) B1->tacc[k] += -fm * ltd[k];
          for (int k = 0; k < 3; ++k) B2->tacc[k] += -fm * ltd[k];
        }
      }
    }
  }
  if (L->limit) {
    real k = info->fps * L->stop_erp;
    info->c[row] = -k * L->limit_err;
    info->cfm[row] = L->stop_cfm;
    if (L->lostop == L->histop) {
      info->lo[row] = -R_INF; info->hi[row] = R_INF;
    } else {
      if (L->limit == 1) { info->lo[row] = 0; info->hi[row] = R_INF; }
      else { info->lo[row] = -R_INF; info->hi[row] = 0; }
      if (L->bounce > 0) {
        real vel;
        if (rotational) {
          vel = dot3(W->body[J->b[0]].avel, ax1);
          if (J->b[1] >= 0) vel -= dot3(W->body[J->b[1]].avel, ax1);
        } else {
          vel = dot3(W->body[J->b[0]].lvel, ax1);
          if (J->b[1] >= 0) vel -= dot3(W->body[J->b[1]].lvel, ax1);
        }
        if (L->limit == 1) {
          if (vel < 0) { real newc = -L->bounce * vel; if (newc > info->c[row]) info->c[row] = newc; }
        } else {
          if (vel > 0) { real newc = -L->bounce * vel; if (newc < info->c[row]) info->c[row] = newc; }
        }
      }
    }
  }
  return 1;
}

/* dJointGetSliderPosition, ode/src/joints/slider.cpp:42-79 */
static real slider_position(OWorld* W, OJoint* J) {
  real ax1[3], q[3];
  const OBody* B1 = &W->body[J->b[0]];
  mul0_331(ax1, B1->R, J->axis1);
  if (J->b[1] >= 0) {
    const OBody* B2 = &W->body[J->b[1]];
    mul0_331(q, B2->R, J->offset);
    for (int i = 0; i < 3; ++i) q[i] = B1->pos[i] - q[i] - B2->pos[i];
  } else {
    for (int i = 0; i < 3; ++i) q[i] = B1->pos[i] - J->offset[i];
    if (J->reverse) { ax1[0] = -ax1[0]; ax1[1] = -ax1[1]; ax1[2] = -ax1[2]; }
  }
  return dot3(ax1, q);
}

/* dxJointUniversal::getAngles, ode/src/joints/universal.cpp:73-167 */
static void universal_angles(OWorld* W, OJoint* J, real* angle1, real* angle2) {
  real ax1[3], ax2[3], qcross[4], qq[4], qrel[4], qcross2[4];
  real R[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  universal_axes(W, J, ax1, ax2);
  r_from_2axes(R, ax1[0], ax1[1], ax1[2], ax2[0], ax2[1], ax2[2]);
  q_from_r(qcross, R);
  qmul1(qq, W->body[J->b[0]].q, qcross);
  qmul2(qrel, qq, J->qrel);
  *angle1 = hinge_angle_from_qrel(qrel, J->axis1);
  qrel[0] = 0;
  qrel[1] = ax1[0] + ax2[0];
  qrel[2] = ax1[1] + ax2[1];
  qrel[3] = ax1[2] + ax2[2];
  real l = 1 / sqrt(qrel[1] * qrel[1] + qrel[2] * qrel[2] + qrel[3] * qrel[3]);
  qrel[1] *= l; qrel[2] *= l; qrel[3] *= l;
  qmul0(qcross2, qrel, qcross);
  if (J->b[1] >= 0) {
    qmul1(qq, W->body[J->b[1]].q, qcross2);
    qmul2(qrel, qq, J->qrel2);
  } else {
    qmul2(qrel, qcross2, J->qrel2);
  }
  *angle2 = -hinge_angle_from_qrel(qrel, J->axis2);
}

/* setFixedOrientation, ode/src/joints/joint.cpp:202-255 */
static void set_fixed_orientation(OWorld* W, OJoint* J, Info2* info, const real* qrel, int start_row) {
  int s = info->rowskip, si = start_row * s;
  info->J1a[si] = 1; info->J1a[si + s + 1] = 1; info->J1a[si + 2 * s + 2] = 1;
  if (J->b[1] >= 0) { info->J2a[si] = -1; info->J2a[si + s + 1] = -1; info->J2a[si + 2 * s + 2] = -1; }
  real qerr[4], e[3];
  if (J->b[1] >= 0) {
    real qq[4];
    qmul1(qq, W->body[J->b[0]].q, W->body[J->b[1]].q);
    qmul2(qerr, qq, qrel);
  } else {
    qmul3(qerr, W->body[J->b[0]].q, qrel);
  }
  if (qerr[0] < 0) { qerr[1] = -qerr[1]; qerr[2] = -qerr[2]; qerr[3] = -qerr[3]; }
  mul0_331(e, W->body[J->b[0]].R, qerr + 1);
  real k = info->fps * info->erp;
  info->c[start_row] = 2 * k * e[0];
  info->c[start_row + 1] = 2 * k * e[1];
  info->c[start_row + 2] = 2 * k * e[2];
}

/* dxJointHinge2::measureAngle, ode/src/joints/hinge2.cpp:33-41 */
static real hinge2_measure_angle(OWorld* W, OJoint* J) {
  real a1[3], a2[3];
  mul0_331(a1, W->body[J->b[1]].R, J->axis2);
  mul1_331(a2, W->body[J->b[0]].R, a1);
  real x = dot3(J->v1, a2);
  real y = dot3(J->v2, a2);
  return -atan2(y, x);
}

/* getInfo1 for each joint type: contact ode/src/joints/contact.cpp:47-71,
 * ball ode/src/joints/ball.cpp:56-60, hinge ode/src/joints/hinge.cpp:54-74,
 * hinge2 ode/src/joints/hinge2.cpp:81-101. Returns m. */
static int joint_info1(OWorld* W, OJoint* J) {
  switch (J->type) {
    case ODEGPU_JOINT_CONTACT: {
      int m = 1;
      odegpuSurface* S = &J->surf;
      if (S->mu < 0) S->mu = 0;
      if (S->mode & ODEGPU_CONTACT_MU2) {
        if ((S->mu > 0) || (S->mu2 > 0)) m++;
        if (S->mu2 < 0) S->mu2 = 0;
        if (S->mu2 > 0) m++;
      } else {
        if (S->mu > 0) m += 2;
      }
      J->the_m = m;
      return m;
    }
    case ODEGPU_JOINT_BALL: return 3;
    case ODEGPU_JOINT_HINGE: {
      int m = (J->lm1.fmax > 0) ? 6 : 5;
      if ((J->lm1.lostop >= -R_PI || J->lm1.histop <= R_PI) && J->lm1.lostop <= J->lm1.histop) {
        real angle = hinge_angle(W, J);
        if (limot_test(&J->lm1, angle)) m = 6;
      }
      return m;
    }
    case ODEGPU_JOINT_HINGE2: {
      int m = 4;
      J->lm1.limit = 0;
      if ((J->lm1.lostop >= -R_PI || J->lm1.histop <= R_PI) && J->lm1.lostop <= J->lm1.histop) {
        real angle = hinge2_measure_angle(W, J);
        limot_test(&J->lm1, angle);
      }
      if (J->lm1.limit || J->lm1.fmax > 0) m++;
      J->lm2.limit = 0;
      if (J->lm2.fmax > 0) m++;
      return m;
    }
    case ODEGPU_JOINT_SLIDER: {
      /* ode/src/joints/slider.cpp:134-167 */
      int m = (J->lm1.fmax > 0) ? 6 : 5;
      J->lm1.limit = 0;
      if ((J->lm1.lostop > -R_INF || J->lm1.histop < R_INF) && J->lm1.lostop <= J->lm1.histop) {
        real pos = slider_position(W, J);
        if (limot_test(&J->lm1, pos)) m = 6;
      }
      return m;
    }
    case ODEGPU_JOINT_UNIVERSAL: {
      /* ode/src/joints/universal.cpp:265-293 */
      int m = 4;
      int lim1 = (J->lm1.lostop >= -R_PI || J->lm1.histop <= R_PI) && J->lm1.lostop <= J->lm1.histop;
      int lim2 = (J->lm2.lostop >= -R_PI || J->lm2.histop <= R_PI) && J->lm2.lostop <= J->lm2.histop;
      J->lm1.limit = 0;
      J->lm2.limit = 0;
      if (lim1 || lim2) {
        real a1, a2;
        universal_angles(W, J, &a1, &a2);
        if (lim1) limot_test(&J->lm1, a1);
        if (lim2) limot_test(&J->lm2, a2);
      }
      if (J->lm1.limit || J->lm1.fmax > 0) m++;
      if (J->lm2.limit || J->lm2.fmax > 0) m++;
      return m;
    }
    case ODEGPU_JOINT_FIXED: return 6;   /* ode/src/joints/fixed.cpp:53-58 */
    case ODEGPU_JOINT_AMOTOR: {
      /* ode/src/joints/amotor.cpp:187-210 */
      int m = 0;
      if (J->am_mode == 1) {
        real ax[3][4];
        amotor_axes(W, J, ax);
        amotor_euler_angles(W, J, ax);
      }
      OLimot* lm[3] = {&J->lm1, &J->lm2, &J->lm3};
      for (int i = 0; i < J->am_num; ++i)
        if (limot_test(lm[i], J->am_angle[i]) || lm[i]->fmax > 0) m++;
      return m;
    }
  }
  return 0;
}

/* getInfo2 for each joint type: contact ode/src/joints/contact.cpp:75-256,
 * ball ode/src/joints/ball.cpp:63-70 (note: it overwrites info->erp, which
 * then carries over to the joints that follow in the same island),
 * hinge ode/src/joints/hinge.cpp:77-149, hinge2 ode/src/joints/hinge2.cpp:109-180. */
static void joint_info2(OWorld* W, OJoint* J, Info2* info) {
  int s = info->rowskip;
  switch (J->type) {
    case ODEGPU_JOINT_CONTACT: {
      int s2 = 2 * s;
      odegpuSurface* S = &J->surf;
      OBody* B1 = &W->body[J->b[0]];
      OBody* B2 = J->b[1] >= 0 ? &W->body[J->b[1]] : 0;
      real normal[4];
      if (J->reverse) { normal[0] = -J->cnormal[0]; normal[1] = -J->cnormal[1]; normal[2] = -J->cnormal[2]; }
      else { normal[0] = J->cnormal[0]; normal[1] = J->cnormal[1]; normal[2] = J->cnormal[2]; }
      normal[3] = 0;
      real c1[3], c2[3] = {0, 0, 0};
      c1[0] = J->cpos[0] - B1->pos[0]; c1[1] = J->cpos[1] - B1->pos[1]; c1[2] = J->cpos[2] - B1->pos[2];
      info->J1l[0] = normal[0]; info->J1l[1] = normal[1]; info->J1l[2] = normal[2];
      cross3(info->J1a, c1, normal);
      if (B2) {
        c2[0] = J->cpos[0] - B2->pos[0]; c2[1] = J->cpos[1] - B2->pos[1]; c2[2] = J->cpos[2] - B2->pos[2];
        info->J2l[0] = -normal[0]; info->J2l[1] = -normal[1]; info->J2l[2] = -normal[2];
        cross3(info->J2a, c2, normal);
        info->J2a[0] = -info->J2a[0]; info->J2a[1] = -info->J2a[1]; info->J2a[2] = -info->J2a[2];
      }
      real erp = info->erp;
      if (S->mode & ODEGPU_CONTACT_SOFT_ERP) erp = S->soft_erp;
      real k = info->fps * erp;
      real depth = J->cdepth - W->min_depth;
      if (depth < 0) depth = 0;
      if (S->mode & ODEGPU_CONTACT_SOFT_CFM) info->cfm[0] = S->soft_cfm;
      real motionN = 0;
      if (S->mode & ODEGPU_CONTACT_MOTIONN) motionN = S->motionN;
      const real pushout = k * depth + motionN;
      info->c[0] = pushout;
      const real maxvel = W->max_vel;
      if (info->c[0] > maxvel) info->c[0] = maxvel;
      if (S->mode & ODEGPU_CONTACT_BOUNCE) {
        real outgoing = dot3(info->J1l, B1->lvel) + dot3(info->J1a, B1->avel);
        if (B2) outgoing += dot3(info->J2l, B2->lvel) + dot3(info->J2a, B2->avel);
        outgoing -= motionN;
        if (S->bounce_vel >= 0 && (-outgoing) > S->bounce_vel) {
          real newc = -S->bounce * outgoing + motionN;
          if (newc > info->c[0]) info->c[0] = newc;
        }
      }
      info->lo[0] = 0;
      info->hi[0] = R_INF;
      real t1[3], t2[3];
      if (J->the_m >= 2) {
        plane_space(normal, t1, t2);
        info->J1l[s + 0] = t1[0]; info->J1l[s + 1] = t1[1]; info->J1l[s + 2] = t1[2];
        cross3(info->J1a + s, c1, t1);
        if (B2) {
          info->J2l[s + 0] = -t1[0]; info->J2l[s + 1] = -t1[1]; info->J2l[s + 2] = -t1[2];
          real* p = info->J2a + s;
          cross3(p, c2, t1); p[0] = -p[0]; p[1] = -p[1]; p[2] = -p[2];
        }
        if (S->mode & ODEGPU_CONTACT_MOTION1) info->c[1] = S->motion1;
        info->lo[1] = -S->mu;
        info->hi[1] = S->mu;
        if (S->mode & ODEGPU_CONTACT_APPROX1_1) info->findex[1] = 0;
        if (S->mode & ODEGPU_CONTACT_SLIP1) info->cfm[1] = S->slip1;
      }
      if (J->the_m >= 3) {
        info->J1l[s2 + 0] = t2[0]; info->J1l[s2 + 1] = t2[1]; info->J1l[s2 + 2] = t2[2];
        cross3(info->J1a + s2, c1, t2);
        if (B2) {
          info->J2l[s2 + 0] = -t2[0]; info->J2l[s2 + 1] = -t2[1]; info->J2l[s2 + 2] = -t2[2];
          real* p = info->J2a + s2;
          cross3(p, c2, t2); p[0] = -p[0]; p[1] = -p[1]; p[2] = -p[2];
        }
        if (S->mode & ODEGPU_CONTACT_MOTION2) info->c[2] = S->motion2;
        if (S->mode & ODEGPU_CONTACT_MU2) { info->lo[2] = -S->mu2; info->hi[2] = S->mu2; }
        else { info->lo[2] = -S->mu; info->hi[2] = S->mu; }
        if (S->mode & ODEGPU_CONTACT_APPROX1_2) info->findex[2] = 0;
        if (S->mode & ODEGPU_CONTACT_SLIP2) info->cfm[2] = S->slip2;
      }
      break;
    }
    case ODEGPU_JOINT_BALL:
      info->erp = J->erp;
      info->cfm[0] = J->cfm; info->cfm[1] = J->cfm; info->cfm[2] = J->cfm;
      set_ball(W, J, info, J->anchor1, J->anchor2);
      break;
    case ODEGPU_JOINT_HINGE: {
      set_ball(W, J, info, J->anchor1, J->anchor2);
      real ax1[3], p[3], q[3];
      mul0_331(ax1, W->body[J->b[0]].R, J->axis1);
      plane_space(ax1, p, q);
      int s3 = 3 * s, s4 = 4 * s;
      info->J1a[s3 + 0] = p[0]; info->J1a[s3 + 1] = p[1]; info->J1a[s3 + 2] = p[2];
      info->J1a[s4 + 0] = q[0]; info->J1a[s4 + 1] = q[1]; info->J1a[s4 + 2] = q[2];
      if (J->b[1] >= 0) {
        info->J2a[s3 + 0] = -p[0]; info->J2a[s3 + 1] = -p[1]; info->J2a[s3 + 2] = -p[2];
        info->J2a[s4 + 0] = -q[0]; info->J2a[s4 + 1] = -q[1]; info->J2a[s4 + 2] = -q[2];
      }
      real ax2[3], b[3];
      if (J->b[1] >= 0) mul0_331(ax2, W->body[J->b[1]].R, J->axis2);
      else { ax2[0] = J->axis2[0]; ax2[1] = J->axis2[1]; ax2[2] = J->axis2[2]; }
      cross3(b, ax1, ax2);
      real k = info->fps * info->erp;
      info->c[3] = k * dot3(b, p);
      info->c[4] = k * dot3(b, q);
      limot_add(W, J, &J->lm1, info, 5, ax1, 1);
      break;
    }
    case ODEGPU_JOINT_HINGE2: {
      real sn, cs, q[4], ax1[4], ax2[4];
      hinge2_axis_info(W, J, ax1, ax2, q, &sn, &cs);
      safe_normalize3(q);
      set_ball2(W, J, info, J->anchor1, J->anchor2, ax1, J->susp_erp);
      int s3 = 3 * s;
      info->J1a[s3 + 0] = q[0]; info->J1a[s3 + 1] = q[1]; info->J1a[s3 + 2] = q[2];
      if (J->b[1] >= 0) { info->J2a[s3 + 0] = -q[0]; info->J2a[s3 + 1] = -q[1]; info->J2a[s3 + 2] = -q[2]; }
      real k = info->fps * info->erp;
      info->c[3] = k * (J->c0 * sn - J->s0 * cs);
      int row = 4 + limot_add(W, J, &J->lm1, info, 4, ax1, 1);
      limot_add(W, J, &J->lm2, info, row, ax2, 1);
      info->cfm[0] = J->susp_cfm;
      break;
    }
    case ODEGPU_JOINT_SLIDER: {
      /* ode/src/joints/slider.cpp:171-246 */
      int s3 = 3 * s, s4 = 4 * s;
      OBody* B1 = &W->body[J->b[0]];
      OBody* B2 = J->b[1] >= 0 ? &W->body[J->b[1]] : 0;
      real c[3] = {0, 0, 0};
      if (B2) for (int i = 0; i < 3; ++i) c[i] = B2->pos[i] - B1->pos[i];
      set_fixed_orientation(W, J, info, J->qrel, 0);
      real ax1[3], p[3], q[3];
      mul0_331(ax1, B1->R, J->axis1);
      plane_space(ax1, p, q);
      if (B2) {
        real t[3];
        cross3(t, c, p);
        for (int i = 0; i < 3; ++i) t[i] *= 0.5;
        for (int i = 0; i < 3; ++i) { info->J1a[s3 + i] = t[i]; info->J2a[s3 + i] = t[i]; }
        cross3(t, c, q);
        for (int i = 0; i < 3; ++i) t[i] *= 0.5;
        for (int i = 0; i < 3; ++i) { info->J1a[s4 + i] = t[i]; info->J2a[s4 + i] = t[i]; }
        for (int i = 0; i < 3; ++i) { info->J2l[s3 + i] = -p[i]; info->J2l[s4 + i] = -q[i]; }
      }
      for (int i = 0; i < 3; ++i) { info->J1l[s3 + i] = p[i]; info->J1l[s4 + i] = q[i]; }
      real k = info->fps * info->erp;
      if (B2) {
        real ofs[3];
        mul0_331(ofs, B2->R, J->offset);
        for (int i = 0; i < 3; ++i) c[i] += ofs[i];
        info->c[3] = k * dot3(p, c);
        info->c[4] = k * dot3(q, c);
      } else {
        real ofs[3];
        for (int i = 0; i < 3; ++i) ofs[i] = J->offset[i] - B1->pos[i];
        info->c[3] = k * dot3(p, ofs);
        info->c[4] = k * dot3(q, ofs);
        if (J->reverse) { ax1[0] = -ax1[0]; ax1[1] = -ax1[1]; ax1[2] = -ax1[2]; }
      }
      limot_add(W, J, &J->lm1, info, 5, ax1, 0);
      break;
    }
    case ODEGPU_JOINT_UNIVERSAL: {
      /* ode/src/joints/universal.cpp:296-362 */
      set_ball(W, J, info, J->anchor1, J->anchor2);
      real ax1[3], ax2[3], t[3], p[3];
      universal_axes(W, J, ax1, ax2);
      real k = dot3(ax1, ax2);
      t[0] = ax2[0] - k * ax1[0];
      t[1] = ax2[1] - k * ax1[1];
      t[2] = ax2[2] - k * ax1[2];
      cross3(p, ax1, t);
      safe_normalize3(p);
      int s3 = 3 * s;
      for (int i = 0; i < 3; ++i) info->J1a[s3 + i] = p[i];
      if (J->b[1] >= 0) for (int i = 0; i < 3; ++i) info->J2a[s3 + i] = -p[i];
      info->c[3] = info->fps * info->erp * -k;
      int row = 4 + limot_add(W, J, &J->lm1, info, 4, ax1, 1);
      limot_add(W, J, &J->lm2, info, row, ax2, 1);
      break;
    }
    case ODEGPU_JOINT_AMOTOR: {
      /* ode/src/joints/amotor.cpp:213-256 */
      real ax[3][4], e0[4], e2[4];
      const real* axp[3];
      amotor_axes(W, J, ax);
      axp[0] = ax[0]; axp[1] = ax[1]; axp[2] = ax[2];
      if (J->am_mode == 1) {
        cross3(e2, ax[0], ax[1]);
        axp[2] = e2;
        cross3(e0, ax[1], ax[2]);
        axp[0] = e0;
      }
      OLimot* lm[3] = {&J->lm1, &J->lm2, &J->lm3};
      int row = 0;
      for (int i = 0; i < J->am_num; ++i) row += limot_add(W, J, lm[i], info, row, axp[i], 1);
      break;
    }
    case ODEGPU_JOINT_FIXED: {
      /* ode/src/joints/fixed.cpp:62-105: the orientation rows use the erp
       * the joint finds in info, then info->erp becomes the joint's own */
      OBody* B1 = &W->body[J->b[0]];
      OBody* B2 = J->b[1] >= 0 ? &W->body[J->b[1]] : 0;
      set_fixed_orientation(W, J, info, J->qrel, 3);
      info->J1l[0] = 1; info->J1l[s + 1] = 1; info->J1l[2 * s + 2] = 1;
      info->erp = J->erp;
      info->cfm[0] = J->cfm; info->cfm[1] = J->cfm; info->cfm[2] = J->cfm;
      real ofs[3];
      mul0_331(ofs, B1->R, J->offset);
      if (B2) {
        /* dSetCrossMatrixPlus(J1a, ofs, s) */
        info->J1a[1] = -ofs[2]; info->J1a[2] = +ofs[1];
        info->J1a[s + 0] = +ofs[2]; info->J1a[s + 2] = -ofs[0];
        info->J1a[2 * s + 0] = -ofs[1]; info->J1a[2 * s + 1] = +ofs[0];
        info->J2l[0] = -1; info->J2l[s + 1] = -1; info->J2l[2 * s + 2] = -1;
      }
      real k = info->fps * info->erp;
      if (B2) for (int j = 0; j < 3; ++j) info->c[j] = k * (B2->pos[j] - B1->pos[j] + ofs[j]);
      else for (int j = 0; j < 3; ++j) info->c[j] = k * (J->offset[j] - B1->pos[j]);
      break;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* SOR_LCP, ode/src/quickstep.cpp:342-584 (WARM_STARTING and               */
/* REORDER_CONSTRAINTS off, RANDOMLY_REORDER_CONSTRAINTS on, :47-64)        */

static void sor_lcp_core(int m, int nb, real* J, const int* jb, const real* invMass, const real* invI,
                         real* lambda, real* fc, real* b, const real* lo, const real* hi,
                         const real* cfm, const int* findex, int num_iterations, real sor_w,
                         real* iMJ_out) {
  memset(lambda, 0, m * sizeof(real));
  real* iMJ = iMJ_out ? iMJ_out : (real*)malloc((size_t)m * 12 * sizeof(real));
  /* compute_invM_JT, :117-136 */
  for (int i = 0; i < m; i++) {
    const real* Jp = J + 12 * i;
    real* ip = iMJ + 12 * i;
    int b1 = jb[2 * i], b2 = jb[2 * i + 1];
    real k1 = invMass[b1];
    for (int j = 0; j < 3; j++) ip[j] = k1 * Jp[j];
    mul0_331(ip + 3, invI + 12 * b1, Jp + 3);
    if (b2 != -1) {
      real k2 = invMass[b2];
      for (int j = 0; j < 3; j++) ip[j + 6] = k2 * Jp[j + 6];
      mul0_331(ip + 9, invI + 12 * b2, Jp + 9);
    }
  }
  memset(fc, 0, (size_t)nb * 6 * sizeof(real));
  real* Ad = (real*)malloc((size_t)m * sizeof(real));
  for (int i = 0; i < m; i++) {
    const real* Jp = J + 12 * i;
    const real* ip = iMJ + 12 * i;
    real sum = 0;
    for (int j = 0; j < 6; j++) sum += ip[j] * Jp[j];
    if (jb[2 * i + 1] != -1)
      for (int k = 6; k < 12; k++) sum += ip[k] * Jp[k];
    Ad[i] = sor_w / (sum + cfm[i]);
  }
  for (int i = 0; i < m; i++) {
    real* Jp = J + 12 * i;
    real Ad_i = Ad[i];
    for (int j = 0; j < 12; j++) Jp[j] *= Ad_i;
    b[i] *= Ad_i;
    Ad[i] = Ad_i * cfm[i];
  }
  int* order = (int*)malloc((size_t)(m > 0 ? m : 1) * sizeof(int));
  {
    int head = 0, tail = m - 1;
    for (int i = 0; i < m; i++) {
      if (findex[i] == -1) order[head++] = i;
      else order[tail--] = i;
    }
  }
  for (int it = 0; it < num_iterations; it++) {
    if ((it & 7) == 0) {
      for (int i = 1; i < m; i++) {
        int swapi = rand_int(i + 1);
        int tmp = order[i];
        order[i] = order[swapi];
        order[swapi] = tmp;
      }
    }
    for (int i = 0; i < m; i++) {
      int index = order[i];
      int b1 = jb[2 * index], b2 = jb[2 * index + 1];
      real* fc1 = fc + 6 * b1;
      real* fc2 = (b2 != -1) ? fc + 6 * b2 : 0;
      real old_lambda = lambda[index];
      real delta = b[index] - old_lambda * Ad[index];
      const real* Jp = J + 12 * index;
      delta -= fc1[0] * Jp[0] + fc1[1] * Jp[1] + fc1[2] * Jp[2] + fc1[3] * Jp[3] + fc1[4] * Jp[4] +
               fc1[5] * Jp[5];
      if (fc2)
        delta -= fc2[0] * Jp[6] + fc2[1] * Jp[7] + fc2[2] * Jp[8] + fc2[3] * Jp[9] + fc2[4] * Jp[10] +
                 fc2[5] * Jp[11];
      real hi_act, lo_act;
      if (findex[index] != -1) {
        hi_act = fabs(hi[index] * lambda[findex[index]]);
        lo_act = -hi_act;
      } else {
        hi_act = hi[index];
        lo_act = lo[index];
      }
      real new_lambda = old_lambda + delta;
      if (new_lambda < lo_act) { delta = lo_act - old_lambda; lambda[index] = lo_act; }
      else if (new_lambda > hi_act) { delta = hi_act - old_lambda; lambda[index] = hi_act; }
      else lambda[index] = new_lambda;
      const real* ip = iMJ + 12 * index;
      fc1[0] += delta * ip[0]; fc1[1] += delta * ip[1]; fc1[2] += delta * ip[2];
      fc1[3] += delta * ip[3]; fc1[4] += delta * ip[4]; fc1[5] += delta * ip[5];
      if (fc2) {
        fc2[0] += delta * ip[6]; fc2[1] += delta * ip[7]; fc2[2] += delta * ip[8];
        fc2[3] += delta * ip[9]; fc2[4] += delta * ip[10]; fc2[5] += delta * ip[11];
      }
    }
  }
  free(order);
  free(Ad);
  if (!iMJ_out) free(iMJ);
}

void oracle_sor_lcp(int m, int nb, double* J, const int* jb, const double* invMass, const double* invI,
                    double* lambda, double* fc, double* b, const double* lo, const double* hi,
                    const double* cfm, const int* findex, int iterations, double sor_w,
                    unsigned int* seed) {
  unsigned int saved = g_seed;
  g_seed = *seed;
  sor_lcp_core(m, nb, J, jb, invMass, invI, lambda, fc, b, lo, hi, cfm, findex, iterations, sor_w, 0);
  *seed = g_seed;
  g_seed = saved;
}

/* ------------------------------------------------------------------------ */
/* dxStepBody, ode/src/util.cpp:255-360 (no finite rotation, no damping,   */
/* no angular speed cap: the defaults on this path)                          */

static void step_body(OBody* b, real h) {
  for (int j = 0; j < 3; j++) b->pos[j] += h * b->lvel[j];
  real dq[4];
  const real* w = b->avel;
  const real* q = b->q;
  dq[0] = 0.5 * (-w[0] * q[1] - w[1] * q[2] - w[2] * q[3]);
  dq[1] = 0.5 * (w[0] * q[0] + w[1] * q[3] - w[2] * q[2]);
  dq[2] = 0.5 * (-w[0] * q[3] + w[1] * q[0] + w[2] * q[1]);
  dq[3] = 0.5 * (w[0] * q[2] - w[1] * q[1] + w[2] * q[0]);
  for (int j = 0; j < 4; j++) b->q[j] += h * dq[j];
  normalize4(b->q);
  r_from_q(b->R, b->q);
}

/* ------------------------------------------------------------------------ */
/* dxQuickStepper, ode/src/quickstep.cpp:592-1025, for one island          */

static void quick_stepper(OWorld* W, const int* bidx, int nb, const int* jidx, int nj_in, real h,
                          int island_no) {
  const real h1 = 1.0 / h;
  real* invI = (real*)malloc((size_t)(nb > 0 ? nb : 1) * 12 * sizeof(real));
  for (int i = 0; i < nb; i++) W->body[bidx[i]].tag = i;
  for (int i = 0; i < nb; i++) {
    OBody* b = &W->body[bidx[i]];
    real tmp[12];
    mul2_333(tmp, b->invI, b->R);
    mul0_333(invI + 12 * i, b->R, tmp);
    if (b->flags & ODEGPU_BODY_GYROSCOPIC) {
      real I[12], t3[3];
      mul2_333(tmp, b->I, b->R);
      mul0_333(I, b->R, tmp);
      mul0_331(t3, I, b->avel);
      real cr[3];
      cross3(cr, b->avel, t3);
      b->tacc[0] = b->tacc[0] - cr[0];
      b->tacc[1] = b->tacc[1] - cr[1];
      b->tacc[2] = b->tacc[2] - cr[2];
    }
  }
  for (int d = 0; d < 3; ++d) {
    real g = W->gravity[d];
    if (g) {
      for (int i = 0; i < nb; i++) {
        OBody* b = &W->body[bidx[i]];
        if ((b->flags & ODEGPU_BODY_NO_GRAVITY) == 0) b->facc[d] += b->mass * g;
      }
    }
  }
  /* getInfo1; joints with m=0 dropped (:670-688) */
  int* jl = (int*)malloc((size_t)(nj_in > 0 ? nj_in : 1) * sizeof(int));
  int* jm = (int*)malloc((size_t)(nj_in > 0 ? nj_in : 1) * sizeof(int));
  int nj = 0, m = 0;
  for (int i = 0; i < nj_in; i++) {
    int mm = joint_info1(W, &W->joint[jidx[i]]);
    if (mm > 0) { jl[nj] = jidx[i]; jm[nj] = mm; nj++; m += mm; }
  }
  W->last_rows += m;
  W->last_islands += m > 0;
  real* cforce = (real*)calloc((size_t)(nb > 0 ? nb : 1) * 6, sizeof(real));
  real *J = 0, *lambda = 0;
  int* jb = 0;
  if (m > 0) {
    J = (real*)calloc((size_t)m * 12, sizeof(real));
    real* cfm = (real*)malloc(m * sizeof(real));
    real* lo = (real*)malloc(m * sizeof(real));
    real* hi = (real*)malloc(m * sizeof(real));
    int* findex = (int*)malloc(m * sizeof(int));
    jb = (int*)malloc((size_t)m * 2 * sizeof(int));
    real* rhs = (real*)malloc(m * sizeof(real));
    real* c = (real*)calloc(m, sizeof(real));
    real* Jcopy = (real*)malloc((size_t)m * 12 * sizeof(real));
    for (int i = 0; i < m; i++) { cfm[i] = W->cfm; lo[i] = -R_INF; hi[i] = R_INF; findex[i] = -1; }
    Info2 info;
    info.rowskip = 12;
    info.fps = h1;
    info.erp = W->erp;
    int ofs = 0;
    for (int k = 0; k < nj; k++) {
      real* Jrow = J + (size_t)ofs * 12;
      info.J1l = Jrow; info.J1a = Jrow + 3; info.J2l = Jrow + 6; info.J2a = Jrow + 9;
      info.c = c + ofs; info.cfm = cfm + ofs; info.lo = lo + ofs; info.hi = hi + ofs;
      info.findex = findex + ofs;
      joint_info2(W, &W->joint[jl[k]], &info);
      memcpy(Jcopy + (size_t)ofs * 12, Jrow, (size_t)jm[k] * 12 * sizeof(real));
      for (int j = 0; j < jm[k]; j++)
        if (findex[ofs + j] != -1) findex[ofs + j] += ofs;
      ofs += jm[k];
    }
    {
      int r = 0;
      for (int k = 0; k < nj; k++) {
        OJoint* Jt = &W->joint[jl[k]];
        int b1 = Jt->b[0] >= 0 ? W->body[Jt->b[0]].tag : -1;
        int b2 = Jt->b[1] >= 0 ? W->body[Jt->b[1]].tag : -1;
        for (int j = 0; j < jm[k]; j++) { jb[2 * r] = b1; jb[2 * r + 1] = b2; r++; }
      }
    }
    {
      real* tmp1 = (real*)malloc((size_t)nb * 6 * sizeof(real));
      for (int i = 0; i < nb; i++) {
        OBody* b = &W->body[bidx[i]];
        real* t = tmp1 + 6 * i;
        for (int j = 0; j < 3; j++) t[j] = b->facc[j] * b->invMass + b->lvel[j] * h1;
        mul0_331(t + 3, invI + 12 * i, b->tacc);
        for (int k = 0; k < 3; k++) t[3 + k] += b->avel[k] * h1;
      }
      /* multiply_J, :163-181 */
      for (int i = 0; i < m; i++) {
        const real* Jp = J + 12 * i;
        int b1 = jb[2 * i], b2 = jb[2 * i + 1];
        real sum = 0;
        const real* in = tmp1 + 6 * b1;
        for (int j = 0; j < 6; j++) sum += Jp[j] * in[j];
        if (b2 != -1) {
          in = tmp1 + 6 * b2;
          for (int j = 0; j < 6; j++) sum += Jp[6 + j] * in[j];
        }
        rhs[i] = sum;
      }
      free(tmp1);
    }
    for (int i = 0; i < m; i++) rhs[i] = c[i] * h1 - rhs[i];
    for (int j = 0; j < m; j++) cfm[j] *= h1;

    lambda = (real*)malloc(m * sizeof(real));
    real* invMass = (real*)malloc((size_t)nb * sizeof(real));
    for (int i = 0; i < nb; i++) invMass[i] = W->body[bidx[i]].invMass;

    oracleTap* tap = W->tap;
    int tap_base = 0;
    if (tap) {
      tap_base = 0;
      for (int q = 0; q < tap->n_islands; ++q) tap_base += tap->island_rows[q];
    }
    if (tap && tap_base + m <= tap->cap_rows) {
      memcpy(tap->J + (size_t)tap_base * 12, J, (size_t)m * 12 * sizeof(real));
      memcpy(tap->rhs + tap_base, rhs, m * sizeof(real));
      memcpy(tap->cfm + tap_base, cfm, m * sizeof(real));
      memcpy(tap->lo + tap_base, lo, m * sizeof(real));
      memcpy(tap->hi + tap_base, hi, m * sizeof(real));
      memcpy(tap->findex + tap_base, findex, m * sizeof(int));
      memcpy(tap->jb + (size_t)tap_base * 2, jb, (size_t)m * 2 * sizeof(int));
      int r = 0;
      for (int k = 0; k < nj; k++)
        for (int j = 0; j < jm[k]; j++) tap->joint_of_row[tap_base + r++] = jl[k];
    }

    sor_lcp_core(m, nb, J, jb, invMass, invI, lambda, cforce, rhs, lo, hi, cfm, findex, W->iterations,
                 W->sor_w, 0);

    if (tap && tap_base + m <= tap->cap_rows) {
      memcpy(tap->lambda + tap_base, lambda, m * sizeof(real));
    }

    for (int i = 0; i < nb; i++) {
      OBody* b = &W->body[bidx[i]];
      for (int j = 0; j < 3; j++) {
        b->lvel[j] += h * cforce[6 * i + j];
        b->avel[j] += h * cforce[6 * i + 3 + j];
      }
    }
    /* joint feedback, :918-957 (Multiply1_12q1) */
    {
      int ofs2 = 0;
      for (int k = 0; k < nj; k++) {
        OJoint* Jt = &W->joint[jl[k]];
        if (Jt->type != ODEGPU_JOINT_CONTACT) {
          for (int half = 0; half < 2; ++half) {
            if (half == 1 && Jt->b[1] < 0) break;
            real a = 0, bb = 0, cc = 0, d = 0, e = 0, f = 0;
            for (int i = 0; i < jm[k]; i++) {
              const real* Bp = Jcopy + (size_t)(ofs2 + i) * 12 + 6 * half;
              real s = lambda[ofs2 + i];
              a += Bp[0] * s; bb += Bp[1] * s; cc += Bp[2] * s;
              d += Bp[3] * s; e += Bp[4] * s; f += Bp[5] * s;
            }
            real* fb = Jt->fb + 6 * half;
            fb[0] = a; fb[1] = bb; fb[2] = cc; fb[3] = d; fb[4] = e; fb[5] = f;
          }
        }
        ofs2 += jm[k];
      }
    }
    free(invMass); free(cfm); free(lo); free(hi); free(findex); free(rhs); free(c); free(Jcopy);
  }
  if (W->tap && W->tap->n_islands < W->tap->cap_islands) {
    oracleTap* tap = W->tap;
    tap->island_rows[tap->n_islands] = m;
    tap->island_bodies[tap->n_islands] = nb;
    int base = 0;
    for (int q = 0; q < tap->n_islands; ++q) base += tap->island_bodies[q];
    if (base + nb <= tap->cap_bodies) {
      for (int i = 0; i < nb; ++i) {
        tap->body_of[base + i] = bidx[i];
        for (int k = 0; k < 6; ++k) tap->cforce[(size_t)(base + i) * 6 + k] = cforce[6 * i + k];
      }
    }
    tap->n_islands++;
  }
  (void)island_no;
  for (int i = 0; i < nb; i++) {
    OBody* b = &W->body[bidx[i]];
    real hm = h * b->invMass;
    for (int j = 0; j < 3; j++) {
      b->lvel[j] += hm * b->facc[j];
      b->tacc[j] *= h;
    }
    real t3[3];
    mul0_331(t3, invI + 12 * i, b->tacc);
    b->avel[0] = b->avel[0] + t3[0];
    b->avel[1] = b->avel[1] + t3[1];
    b->avel[2] = b->avel[2] + t3[2];
  }
  for (int i = 0; i < nb; i++) step_body(&W->body[bidx[i]], h);
  for (int i = 0; i < nb; i++) {
    OBody* b = &W->body[bidx[i]];
    b->facc[0] = b->facc[1] = b->facc[2] = 0;
    b->tacc[0] = b->tacc[1] = b->tacc[2] = 0;
  }
  free(J); free(jb); free(lambda); free(cforce); free(jl); free(jm); free(invI);
}

/* ------------------------------------------------------------------------ */
/* dWorldStep: the exact stepper (ode/src/step.cpp:187-846) with the Dantzig */
/* LCP solver (ode/src/lcp.cpp:360-1073) and the LDL^T kernels it calls      */
/* (ode/src/fastldlt.c, fastlsolve.c, fastltsolve.c, fastdot.c,              */
/* ode/src/matrix.cpp:242-436). The blocked kernels are restated with the    */
/* reference's accumulation order (sums over earlier columns first, then the */
/* terms inside the 2- or 4-row block), which is what makes this FP64        */
/* restatement agree with the reference bit for bit.                         */

/* info->nub of each joint's getInfo1 (ball.cpp:52, hinge.cpp:56,
 * hinge2.cpp:84, slider.cpp:118, universal.cpp:267, fixed.cpp:54,
 * amotor.cpp:194, contact.cpp:51-70); J->the_m / limits set by joint_info1. */
static int joint_nub(const OJoint* J) {
  switch (J->type) {
    case ODEGPU_JOINT_CONTACT: {
      const odegpuSurface* S = &J->surf;
      int nub = 0;
      if (S->mode & ODEGPU_CONTACT_MU2) {
        if (S->mu == R_INF) nub++;
        if (S->mu2 == R_INF) nub++;
      } else if (S->mu == R_INF) {
        nub += 2;
      }
      return nub;
    }
    case ODEGPU_JOINT_BALL: return 3;
    case ODEGPU_JOINT_HINGE: return 5;
    case ODEGPU_JOINT_HINGE2: return 4;
    case ODEGPU_JOINT_SLIDER: return 5;
    case ODEGPU_JOINT_UNIVERSAL: return 4;
    case ODEGPU_JOINT_FIXED: return 6;
    default: return 0;
  }
}

static real lcp_dot(const real* a, const real* b, int n) {   /* _dDot, fastdot.c */
  real sum = 0;
  for (int k = 0; k < n; ++k) sum += a[k] * b[k];
  return sum;
}

/* Unit lower-triangular solve in blocks of 4 rows (_dSolveL1, fastlsolve.c;
 * _dSolveL1T, fastltsolve.c, is the same on the reversed transposed system).
 * M(r, c) is the matrix entry of row r, column c < r in processing order;
 * x is indexed in processing order too. */
#define LSOLVE_BLOCKED(n, M, X)                                                              \
  do {                                                                                        \
    int i_ = 0;                                                                               \
    for (; i_ <= (n) - 4; i_ += 4) {                                                          \
      real z_[4] = {0, 0, 0, 0};                                                              \
      for (int c_ = 0; c_ < i_; ++c_)                                                         \
        for (int q_ = 0; q_ < 4; ++q_) z_[q_] += M(i_ + q_, c_) * X(c_);                      \
      real v0 = X(i_) - z_[0];                                                                \
      X(i_) = v0;                                                                             \
      real v1 = X(i_ + 1) - z_[1] - M(i_ + 1, i_) * v0;                                       \
      X(i_ + 1) = v1;                                                                         \
      real v2 = X(i_ + 2) - z_[2] - M(i_ + 2, i_) * v0 - M(i_ + 2, i_ + 1) * v1;             \
      X(i_ + 2) = v2;                                                                         \
      X(i_ + 3) = X(i_ + 3) - z_[3] - M(i_ + 3, i_) * v0 - M(i_ + 3, i_ + 1) * v1 -           \
                  M(i_ + 3, i_ + 2) * v2;                                                     \
    }                                                                                         \
    for (; i_ < (n); ++i_) {                                                                  \
      real z0 = 0;                                                                            \
      for (int c_ = 0; c_ < i_; ++c_) z0 += M(i_, c_) * X(c_);                                \
      X(i_) = X(i_) - z0;                                                                     \
    }                                                                                         \
  } while (0)

static void lcp_solve_l1(const real* L, real* B, int n, int ns) {
#define ML(r, c) L[(size_t)(r) * ns + (c)]
#define XB(i) B[i]
  LSOLVE_BLOCKED(n, ML, XB);
#undef ML
#undef XB
}
static void lcp_solve_l1t(const real* L, real* B, int n, int ns) {
#define MLT(r, c) L[(size_t)(n - 1 - (c)) * ns + (n - 1 - (r))]
#define XBT(i) B[n - 1 - (i)]
  LSOLVE_BLOCKED(n, MLT, XBT);
#undef MLT
#undef XBT
}

/* dSolveL1_1 / dSolveL1_2 of fastldlt.c: blocks of 2 rows, one or two right
 * hand sides (rows of A, B1 / B2 stored at stride 1). */
static void lcp_solve_l1_pair(const real* L, real* B1, real* B2, int n, int ns) {
  for (int i = 0; i < n; i += 2) {
    real z11 = 0, z12 = 0, z21 = 0, z22 = 0;
    for (int c = 0; c < i; ++c) {
      const real p1 = L[(size_t)i * ns + c], p2 = L[(size_t)(i + 1) * ns + c];
      z11 += p1 * B1[c];
      if (B2) z12 += p1 * B2[c];
      z21 += p2 * B1[c];
      if (B2) z22 += p2 * B2[c];
    }
    const real l = L[(size_t)(i + 1) * ns + i];
    z11 = B1[i] - z11;
    B1[i] = z11;
    if (B2) { z12 = B2[i] - z12; B2[i] = z12; }
    B1[i + 1] = B1[i + 1] - z21 - l * z11;
    if (B2) B2[i + 1] = B2[i + 1] - z22 - l * z12;
  }
}

/* _dFactorLDLT (fastldlt.c): A = L D L^T in place (L below the diagonal),
 * d = 1 / D, two rows at a time. */
static void lcp_factor_ldlt(real* A, real* d, int n, int ns) {
  if (n < 1) return;
  int i = 0;
  for (; i <= n - 2; i += 2) {
    real* r1 = A + (size_t)i * ns;
    real* r2 = A + (size_t)(i + 1) * ns;
    lcp_solve_l1_pair(A, r1, r2, i, ns);
    real z11 = 0, z21 = 0, z22 = 0;
    for (int j = 0; j < i; ++j) {
      const real p1 = r1[j], p2 = r2[j], dd = d[j];
      const real q1 = p1 * dd, q2 = p2 * dd;
      r1[j] = q1;
      r2[j] = q2;
      z11 += p1 * q1;
      z21 += p2 * q1;
      z22 += p2 * q2;
    }
    z11 = r1[i] - z11;
    z21 = r2[i] - z21;
    z22 = r2[i + 1] - z22;
    d[i] = 1.0 / z11;
    const real q1 = z21, q2 = q1 * d[i];
    d[i + 1] = 1.0 / (z22 - q1 * q2);
    r2[i] = q2;
  }
  if (n - i == 1) {
    real* r1 = A + (size_t)i * ns;
    lcp_solve_l1_pair(A, r1, NULL, i, ns);
    real z11 = 0;
    for (int j = 0; j < i; ++j) {
      const real p1 = r1[j], q1 = p1 * d[j];
      r1[j] = q1;
      z11 += p1 * q1;
    }
    d[i] = 1.0 / (r1[i] - z11);
  }
}

static void lcp_solve_ldlt(const real* L, const real* d, real* b, int n, int ns) {   /* matrix.cpp:251-257 */
  lcp_solve_l1(L, b, n, ns);
  for (int i = 0; i < n; ++i) b[i] *= d[i];
  lcp_solve_l1t(L, b, n, ns);
}

/* _dLDLTAddTL, matrix.cpp:260-336: rank-2 update of the factorization for
 * the top-left row / column replaced by a. */
static void lcp_ldlt_add_tl(real* L, real* d, const real* a, int n, int ns, real* W1, real* W2) {
  if (n < 2) return;
  W1[0] = W2[0] = 0;
  for (int j = 1; j < n; ++j) W1[j] = W2[j] = a[j] * M_SQRT1_2;
  const real W11 = (0.5 * a[0] + 1) * M_SQRT1_2;
  const real W21 = (0.5 * a[0] - 1) * M_SQRT1_2;
  real alpha1 = 1.0, alpha2 = 1.0;
  {
    real dee = d[0];
    real alphanew = alpha1 + (W11 * W11) * dee;
    dee /= alphanew;
    const real gamma1 = W11 * dee;
    dee *= alpha1;
    alpha1 = alphanew;
    alphanew = alpha2 - (W21 * W21) * dee;
    dee /= alphanew;
    alpha2 = alphanew;
    const real k1 = 1.0 - W21 * gamma1;
    const real k2 = W21 * gamma1 * W11 - W21;
    for (int p = 1; p < n; ++p) {
      const real Wp = W1[p], ell = L[(size_t)p * ns];
      W1[p] = Wp - W11 * ell;
      W2[p] = k1 * Wp + k2 * ell;
    }
  }
  for (int j = 1; j < n; ++j) {
    const real k1 = W1[j], k2 = W2[j];
    real dee = d[j];
    real alphanew = alpha1 + (k1 * k1) * dee;
    dee /= alphanew;
    const real gamma1 = k1 * dee;
    dee *= alpha1;
    alpha1 = alphanew;
    alphanew = alpha2 - (k2 * k2) * dee;
    dee /= alphanew;
    const real gamma2 = k2 * dee;
    dee *= alpha2;
    d[j] = dee;
    alpha2 = alphanew;
    for (int p = j + 1; p < n; ++p) {
      real* l = &L[(size_t)p * ns + j];
      real ell = *l;
      real Wp = W1[p] - k1 * ell;
      ell += gamma1 * Wp;
      W1[p] = Wp;
      Wp = W2[p] - k2 * ell;
      ell -= gamma2 * Wp;
      W2[p] = Wp;
      *l = ell;
    }
  }
}

/* Dantzig LCP state (the dLCP object, lcp.cpp:362-785), rows of A reached
 * through row pointers so that row swaps exchange pointers. */
typedef struct {
  int n, ns, nub, nC, nN;
  real** A;
  real *x, *b, *w, *lo, *hi, *L, *d, *Dell, *ell, *tmp, *W1, *W2, *t;
  int *state, *findex, *p, *C;
} LcpState;

#define LCP_GETA(S, i, j) (((i) > (j)) ? (S)->A[i][j] : (S)->A[j][i])

/* swapRowsAndCols (lcp.cpp:148-213, row-pointer variant) */
static void lcp_swap_rows_cols(LcpState* S, int i1, int i2, int fast) {
  real** A = S->A;
  real* A_i1 = A[i1];
  real* A_i2 = A[i2];
  for (int i = i1 + 1; i < i2; ++i) {
    real* A_i_i1 = A[i] + i1;
    A_i1[i] = *A_i_i1;
    *A_i_i1 = A_i2[i];
  }
  A_i1[i2] = A_i1[i1];
  A_i1[i1] = A_i2[i1];
  A_i2[i1] = A_i2[i2];
  if (fast) {
    A[i1] = A_i2;
    A[i2] = A_i1;
  } else {
    for (int k = 0; k <= i2; ++k) { const real t = A_i1[k]; A_i1[k] = A_i2[k]; A_i2[k] = t; }
  }
  for (int j = i2 + 1; j < S->n; ++j) {
    real* A_j = A[j];
    const real t = A_j[i1]; A_j[i1] = A_j[i2]; A_j[i2] = t;
  }
}

/* swapProblem (lcp.cpp:216-267) */
static void lcp_swap_problem(LcpState* S, int i1, int i2, int fast) {
  if (i1 == i2) return;
  lcp_swap_rows_cols(S, i1, i2, fast);
#define SWPR(v) { const real t_ = S->v[i1]; S->v[i1] = S->v[i2]; S->v[i2] = t_; }
#define SWPI(v) { const int t_ = S->v[i1]; S->v[i1] = S->v[i2]; S->v[i2] = t_; }
  SWPR(x) SWPR(b) SWPR(w) SWPR(lo) SWPR(hi) SWPI(p) SWPI(state)
  if (S->findex) SWPI(findex)
#undef SWPR
#undef SWPI
}

static void lcp_transfer_i_to_C(LcpState* S, int i) {   /* lcp.cpp:524-551 */
  if (S->nC > 0) {
    real* Lt = S->L + (size_t)S->nC * S->ns;
    for (int j = 0; j < S->nC; ++j) Lt[j] = S->ell[j];
    S->d[S->nC] = 1.0 / (S->A[i][i] - lcp_dot(S->ell, S->Dell, S->nC));
  } else {
    S->d[0] = 1.0 / S->A[i][i];
  }
  lcp_swap_problem(S, S->nC, i, 1);
  S->C[S->nC] = S->nC;
  S->nC++;
}

static void lcp_gather_dell(LcpState* S, int i) {   /* Dell = A(i, C), NUB_OPTIMIZATIONS */
  const real* aptr = S->A[i];
  int j = 0;
  for (; j < S->nub; ++j) S->Dell[j] = aptr[j];
  for (; j < S->nC; ++j) S->Dell[j] = aptr[S->C[j]];
}

static void lcp_transfer_i_from_N_to_C(LcpState* S, int i) {   /* lcp.cpp:555-605 */
  if (S->nC > 0) {
    lcp_gather_dell(S, i);
    lcp_solve_l1(S->L, S->Dell, S->nC, S->ns);
    real* Lt = S->L + (size_t)S->nC * S->ns;
    for (int j = 0; j < S->nC; ++j) Lt[j] = S->ell[j] = S->Dell[j] * S->d[j];
    S->d[S->nC] = 1.0 / (S->A[i][i] - lcp_dot(S->ell, S->Dell, S->nC));
  } else {
    S->d[0] = 1.0 / S->A[i][i];
  }
  lcp_swap_problem(S, S->nC, i, 1);
  S->C[S->nC] = S->nC;
  S->nN--;
  S->nC++;
}

/* _dRemoveRowCol, matrix.cpp:402-434 */
static void lcp_remove_row_col(real* A, int n, int ns, int r) {
  if (r >= n - 1) return;
  if (r > 0) {
    for (int i = 0; i < r; ++i) memmove(A + (size_t)i * ns + r, A + (size_t)i * ns + r + 1, (n - r - 1) * sizeof(real));
    for (int i = r; i < n - 1; ++i) memcpy(A + (size_t)i * ns, A + (size_t)(i + 1) * ns, r * sizeof(real));
  }
  for (int i = r; i < n - 1; ++i)
    memcpy(A + (size_t)i * ns + r, A + (size_t)(i + 1) * ns + r + 1, (n - r - 1) * sizeof(real));
}

/* _dLDLTRemove, matrix.cpp:348-399: drop row / column r of the factorized
 * set C (indices p into A) */
static void lcp_ldlt_remove(LcpState* S, const int* p, int n2, int r) {
  real* L = S->L;
  real* d = S->d;
  const int ns = S->ns;
  if (r == n2 - 1) return;
  if (r == 0) {
    real* a = S->t;
    const int p0 = p[0];
    for (int i = 0; i < n2; ++i) a[i] = -LCP_GETA(S, p[i], p0);
    a[0] += 1.0;
    lcp_ldlt_add_tl(L, d, a, n2, ns, S->W1, S->W2);
  } else {
    real* t = S->t;
    const real* Lr = L + (size_t)r * ns;
    for (int i = 0; i < r; ++i) t[i] = Lr[i] / d[i];
    real* a = t + r;
    const int p_r = p[r];
    for (int i = 0; i < n2 - r; ++i) a[i] = lcp_dot(L + (size_t)(r + i) * ns, t, r) - LCP_GETA(S, p[r + i], p_r);
    a[0] += 1.0;
    lcp_ldlt_add_tl(L + (size_t)r * ns + r, d + r, a, n2 - r, ns, S->W1, S->W2);
  }
  lcp_remove_row_col(L, n2, ns, r);
  if (r < n2 - 1) memmove(d + r, d + r + 1, (n2 - r - 1) * sizeof(real));
}

static void lcp_transfer_i_from_C_to_N(LcpState* S, int i) {   /* lcp.cpp:609-651 */
  int* C = S->C;
  const int nC = S->nC;
  int last_idx = -1, j = 0;
  for (; j < nC; ++j) {
    if (C[j] == nC - 1) last_idx = j;
    if (C[j] == i) {
      lcp_ldlt_remove(S, C, nC, j);
      int k;
      if (last_idx == -1) {
        for (k = j + 1; k < nC; ++k)
          if (C[k] == nC - 1) break;
      } else {
        k = last_idx;
      }
      C[k] = C[j];
      if (j < nC - 1) memmove(C + j, C + j + 1, (nC - j - 1) * sizeof(int));
      break;
    }
  }
  lcp_swap_problem(S, i, nC - 1, 1);
  S->nN++;
  S->nC = nC - 1;
}

/* solve1 (lcp.cpp:704-757): a(C) = -dir A(C,C) \ A(C,i) */
static void lcp_solve1(LcpState* S, real* a, int i, int dir, int only_transfer) {
  if (S->nC <= 0) return;
  lcp_gather_dell(S, i);
  lcp_solve_l1(S->L, S->Dell, S->nC, S->ns);
  for (int j = 0; j < S->nC; ++j) S->ell[j] = S->Dell[j] * S->d[j];
  if (!only_transfer) {
    for (int j = 0; j < S->nC; ++j) S->tmp[j] = S->ell[j];
    lcp_solve_l1t(S->L, S->tmp, S->nC, S->ns);
    if (dir > 0)
      for (int j = 0; j < S->nC; ++j) a[S->C[j]] = -S->tmp[j];
    else
      for (int j = 0; j < S->nC; ++j) a[S->C[j]] = S->tmp[j];
  }
}

/* dSolveLCP (lcp.cpp:784-1073). A is n x ns, row-major, lower triangle used;
 * it is destroyed. Returns 0, or 1 when the solver stopped on s <= 0. */
static int solve_lcp(int n, real* A, real* x, real* b, int nub, real* lo, real* hi, int* findex) {
  const int ns = n;
  if (nub >= n) {
    real* d = (real*)calloc(n, sizeof(real));
    lcp_factor_ldlt(A, d, n, ns);
    lcp_solve_ldlt(A, d, b, n, ns);
    memcpy(x, b, n * sizeof(real));
    free(d);
    return 0;
  }
  LcpState S_, *S = &S_;
  memset(S, 0, sizeof(*S));
  S->n = n; S->ns = ns; S->nub = nub;
  S->A = (real**)malloc(n * sizeof(real*));
  for (int k = 0; k < n; ++k) S->A[k] = A + (size_t)k * ns;
  S->x = x; S->b = b; S->lo = lo; S->hi = hi; S->findex = findex;
  real* buf = (real*)calloc((size_t)n * ns + 12 * (size_t)n + 8, sizeof(real));
  S->L = buf;
  S->d = S->L + (size_t)n * ns;
  S->w = S->d + n; S->Dell = S->w + n; S->ell = S->Dell + n; S->tmp = S->ell + n;
  real* delta_x = S->tmp + n;
  S->W1 = delta_x + n; S->W2 = S->W1 + n; S->t = S->W2 + n;
  real* delta_w = S->tmp;   /* tmp doubles as delta_w (lcp.cpp:835-836) */
  S->state = (int*)calloc(n, sizeof(int));
  S->p = (int*)malloc(n * sizeof(int));
  S->C = (int*)malloc(n * sizeof(int));
  /* dLCP::dLCP, lcp.cpp:400-520 */
  for (int k = 0; k < n; ++k) { x[k] = 0; S->p[k] = k; }
  for (int k = S->nub; k < n; ++k) {
    if (findex && findex[k] >= 0) continue;
    if (lo[k] == -R_INF && hi[k] == R_INF) {
      lcp_swap_problem(S, S->nub, k, 0);
      S->nub++;
    }
  }
  if (S->nub > 0) {
    for (int j = 0; j < S->nub; ++j) memcpy(S->L + (size_t)j * ns, S->A[j], (j + 1) * sizeof(real));
    lcp_factor_ldlt(S->L, S->d, S->nub, ns);
    memcpy(x, b, S->nub * sizeof(real));
    lcp_solve_ldlt(S->L, S->d, x, S->nub, ns);
    for (int k = 0; k < S->nub; ++k) { S->w[k] = 0; S->C[k] = k; }
    S->nC = S->nub;
  }
  if (findex) {
    int at_end = 0;
    for (int k = n - 1; k >= S->nub; k--)
      if (findex[k] >= 0) {
        lcp_swap_problem(S, k, n - 1 - at_end, 1);
        at_end++;
      }
  }
  const int adj_nub = S->nub;
  real* w = S->w;
  int hit_first_friction = 0, err = 0;
  for (int i = adj_nub; i < n; ++i) {
    int s_error = 0;
    if (!hit_first_friction && findex && findex[i] >= 0) {
      for (int j = 0; j < n; ++j) delta_w[S->p[j]] = x[j];
      for (int k = i; k < n; ++k) {
        const real wfk = delta_w[findex[k]];
        if (wfk == 0) { hi[k] = 0; lo[k] = 0; }
        else { hi[k] = fabs(hi[k] * wfk); lo[k] = -hi[k]; }
      }
      hit_first_friction = 1;
    }
    w[i] = lcp_dot(S->A[i], x, S->nC) + lcp_dot(S->A[i] + S->nC, x + S->nC, S->nN) - b[i];
    if (lo[i] == 0 && w[i] >= 0) {
      S->nN++;
      S->state[i] = 0;
    } else if (hi[i] == 0 && w[i] <= 0) {
      S->nN++;
      S->state[i] = 1;
    } else if (w[i] == 0) {
      lcp_solve1(S, delta_x, i, 0, 1);
      lcp_transfer_i_to_C(S, i);
    } else {
      for (;;) {
        int dir;
        real dirf;
        if (w[i] <= 0) { dir = 1; dirf = 1.0; }
        else { dir = -1; dirf = -1.0; }
        lcp_solve1(S, delta_x, i, dir, 0);
        {   /* delta_w(N) = A(N,C) delta_x(C), then += dir A(N,i) */
          const int nC = S->nC, nN = S->nN;
          for (int k = 0; k < nN; ++k) delta_w[nC + k] = lcp_dot(S->A[k + nC], delta_x, nC);
          const real* aptr = S->A[i] + nC;
          if (dir > 0) for (int k = 0; k < nN; ++k) delta_w[nC + k] += aptr[k];
          else for (int k = 0; k < nN; ++k) delta_w[nC + k] -= aptr[k];
        }
        delta_w[i] = lcp_dot(S->A[i], delta_x, S->nC) + S->A[i][i] * dirf;
        int cmd = 1, si = 0;
        real s = -w[i] / delta_w[i];
        if (dir > 0) {
          if (hi[i] < R_INF) {
            const real s2 = (hi[i] - x[i]) * dirf;
            if (s2 < s) { s = s2; cmd = 3; }
          }
        } else {
          if (lo[i] > -R_INF) {
            const real s2 = (lo[i] - x[i]) * dirf;
            if (s2 < s) { s = s2; cmd = 2; }
          }
        }
        for (int k = 0; k < S->nN; ++k) {
          const int ik = S->nC + k;
          if (!S->state[ik] ? delta_w[ik] < 0 : delta_w[ik] > 0) {
            if (lo[ik] == 0 && hi[ik] == 0) continue;
            const real s2 = -w[ik] / delta_w[ik];
            if (s2 < s) { s = s2; cmd = 4; si = ik; }
          }
        }
        for (int k = adj_nub; k < S->nC; ++k) {
          if (delta_x[k] < 0 && lo[k] > -R_INF) {
            const real s2 = (lo[k] - x[k]) / delta_x[k];
            if (s2 < s) { s = s2; cmd = 5; si = k; }
          }
          if (delta_x[k] > 0 && hi[k] < R_INF) {
            const real s2 = (hi[k] - x[k]) / delta_x[k];
            if (s2 < s) { s = s2; cmd = 6; si = k; }
          }
        }
        if (s <= 0.0) {
          for (int k = i; k < n; ++k) { x[k] = 0; w[k] = 0; }
          s_error = 1;
          break;
        }
        for (int k = 0; k < S->nC; ++k) x[k] += s * delta_x[k];
        x[i] += s * dirf;
        for (int k = 0; k < S->nN; ++k) w[S->nC + k] += s * delta_w[S->nC + k];
        w[i] += s * delta_w[i];
        switch (cmd) {
          case 1: w[i] = 0; lcp_transfer_i_to_C(S, i); break;
          case 2: x[i] = lo[i]; S->state[i] = 0; S->nN++; break;
          case 3: x[i] = hi[i]; S->state[i] = 1; S->nN++; break;
          case 4: w[si] = 0; lcp_transfer_i_from_N_to_C(S, si); break;
          case 5: x[si] = lo[si]; S->state[si] = 0; lcp_transfer_i_from_C_to_N(S, si); break;
          case 6: x[si] = hi[si]; S->state[si] = 1; lcp_transfer_i_from_C_to_N(S, si); break;
        }
        if (cmd <= 3) break;
      }
    }
    if (s_error) { err = 1; break; }
  }
  /* unpermute (lcp.cpp:759-781) */
  memcpy(S->tmp, x, n * sizeof(real));
  for (int j = 0; j < n; ++j) x[S->p[j]] = S->tmp[j];
  memcpy(S->tmp, w, n * sizeof(real));
  for (int j = 0; j < n; ++j) w[S->p[j]] = S->tmp[j];
  free(S->A); free(buf); free(S->state); free(S->p); free(S->C);
  return err;
}

typedef struct { int j, m, nub; } JInfo1;

/* The joint order of step.cpp:265-403: purely unbounded joints first, then
 * mixed, then purely LCP ones, built by the reference's two-ended scheme
 * (joints are placed alternately growing forward and backward from the middle
 * of a 2 nj buffer, swapping a mixed joint into place when a group boundary
 * moves). Joints with m = 0 are dropped. Returns the joint count; *nub_out is
 * the number of purely unbounded joints, which the reference passes to the
 * LCP as its nub. */
static int exact_joint_order(OWorld* W, const int* jidx, int nj_in, JInfo1* out, int* nub_out) {
  JInfo1* a = (JInfo1*)malloc((size_t)(2 * nj_in + 2) * sizeof(JInfo1));
  int unb_start, mix_start, mix_end, lcp_end;
  unb_start = mix_start = mix_end = lcp_end = nj_in;
  int cur = lcp_end, src = 0;
  for (;;) {
    int fwd_end = 0;
    {
      int mixend = mix_end;
      for (;;) {
        if (src == nj_in) { lcp_end = cur; fwd_end = 1; break; }
        OJoint* J = &W->joint[jidx[src++]];
        JInfo1 in = {(int)(J - W->joint), joint_info1(W, J), 0};
        in.nub = joint_nub(J);
        if (in.m > 0) {
          if (in.nub == 0) {
            a[cur++] = in;
          } else if (in.nub < in.m) {
            if (unb_start == mix_start) {
              unb_start = mix_start = mix_start - 1;
              a[mix_start] = in;
            } else if (mixend != cur) {
              a[cur] = a[mixend];
              a[mixend] = in;
              ++mixend; ++cur;
            } else {
              a[cur] = in;
              mixend = cur = cur + 1;
            }
          } else {
            unb_start = unb_start - 1;
            a[unb_start] = in;
            lcp_end = cur;
            mix_end = mixend;
            cur = unb_start - 1;
            break;
          }
        }
      }
    }
    if (fwd_end) break;
    int bkw_end = 0;
    {
      int mixstart = mix_start - 1;
      for (;;) {
        if (src == nj_in) { unb_start = cur + 1; mix_start = mixstart + 1; bkw_end = 1; break; }
        OJoint* J = &W->joint[jidx[src++]];
        JInfo1 in = {(int)(J - W->joint), joint_info1(W, J), 0};
        in.nub = joint_nub(J);
        if (in.m > 0) {
          if (in.nub == in.m) {
            a[cur--] = in;
          } else if (in.nub > 0) {
            if (mix_end == lcp_end) {
              const int e = mix_end;
              lcp_end = mix_end = mix_end + 1;
              a[e] = in;
            } else if (mixstart != cur) {
              a[cur] = a[mixstart];
              a[mixstart] = in;
              --mixstart; --cur;
            } else {
              a[cur] = in;
              mixstart = cur = cur - 1;
            }
          } else {
            const int e = lcp_end;
            lcp_end = lcp_end + 1;
            a[e] = in;
            unb_start = cur + 1;
            mix_start = mixstart + 1;
            cur = e + 1;
            break;
          }
        }
      }
    }
    if (bkw_end) break;
  }
  *nub_out = mix_start - unb_start;
  const int nj = lcp_end - unb_start;
  memcpy(out, a + unb_start, (size_t)nj * sizeof(JInfo1));
  free(a);
  return nj;
}

static int g_lcp_errors = 0;   /* LCP runs that stopped on s <= 0 */
static int g_exact_stepper = 0;   /* 1: worlds step with dWorldStep instead of dWorldQuickStep */
void oracle_set_stepper(int exact) { g_exact_stepper = exact; }
int oracle_lcp_errors(void) { return g_lcp_errors; }

static void exact_stepper(OWorld* W, const int* bidx, int nb, const int* jidx, int nj_in, real h) {
  const real h1 = 1.0 / h;
  real* invI = (real*)malloc((size_t)(nb > 0 ? nb : 1) * 12 * sizeof(real));
  for (int i = 0; i < nb; i++) W->body[bidx[i]].tag = i;
  for (int i = 0; i < nb; i++) {   /* step.cpp:205-229 */
    OBody* b = &W->body[bidx[i]];
    real tmp[12];
    mul2_333(tmp, b->invI, b->R);
    mul0_333(invI + 12 * i, b->R, tmp);
    if (b->flags & ODEGPU_BODY_GYROSCOPIC) {
      real I[12], t3[3], cr[3];
      mul2_333(tmp, b->I, b->R);
      mul0_333(I, b->R, tmp);
      mul0_331(t3, I, b->avel);
      cross3(cr, b->avel, t3);
      b->tacc[0] = b->tacc[0] - cr[0];
      b->tacc[1] = b->tacc[1] - cr[1];
      b->tacc[2] = b->tacc[2] - cr[2];
    }
  }
  for (int d = 0; d < 3; ++d) {   /* :231-262 */
    const real g = W->gravity[d];
    if (g)
      for (int i = 0; i < nb; i++) {
        OBody* b = &W->body[bidx[i]];
        if ((b->flags & ODEGPU_BODY_NO_GRAVITY) == 0) b->facc[d] += b->mass * g;
      }
  }
  JInfo1* ji = (JInfo1*)malloc((size_t)(nj_in > 0 ? nj_in : 1) * sizeof(JInfo1));
  int nub = 0;
  const int nj = exact_joint_order(W, jidx, nj_in, ji, &nub);
  int m = 0;
  int* ofs = (int*)malloc((size_t)(nj > 0 ? nj : 1) * sizeof(int));
  for (int k = 0; k < nj; ++k) { ofs[k] = m; m += ji[k].m; }
  W->last_rows += m;
  W->last_islands += m > 0;
  real* cforce = (real*)calloc((size_t)(nb > 0 ? nb : 1) * 6, sizeof(real));
  if (m > 0) {
    real* lo = (real*)malloc(m * sizeof(real));
    real* hi = (real*)malloc(m * sizeof(real));
    real* J = (real*)calloc((size_t)m * 12, sizeof(real));
    real* JinvM = (real*)calloc((size_t)m * 12, sizeof(real));
    int* findex = (int*)malloc(m * sizeof(int));
    real* A = (real*)calloc((size_t)m * m, sizeof(real));
    real* rhs = (real*)calloc(m, sizeof(real));   /* c, then rhs */
    real* cfm = (real*)malloc(m * sizeof(real));
    int* jb = (int*)malloc((size_t)nj * 2 * sizeof(int));
    for (int i = 0; i < m; ++i) { lo[i] = -R_INF; hi[i] = R_INF; findex[i] = -1; cfm[i] = W->cfm; }
    /* create J (:457-497) */
    Info2 info;
    info.rowskip = 12;
    info.fps = h1;
    info.erp = W->erp;
    for (int k = 0; k < nj; ++k) {
      real* Jrow = J + (size_t)ofs[k] * 12;
      info.J1l = Jrow; info.J1a = Jrow + 3; info.J2l = Jrow + 6; info.J2a = Jrow + 9;
      info.c = rhs + ofs[k]; info.cfm = cfm + ofs[k]; info.lo = lo + ofs[k]; info.hi = hi + ofs[k];
      info.findex = findex + ofs[k];
      OJoint* Jt = &W->joint[ji[k].j];
      joint_info2(W, Jt, &info);
      for (int r = 0; r < ji[k].m; ++r)
        if (findex[ofs[k] + r] != -1) findex[ofs[k] + r] += ofs[k];
      jb[2 * k] = Jt->b[0] >= 0 ? W->body[Jt->b[0]].tag : -1;
      jb[2 * k + 1] = Jt->b[1] >= 0 ? W->body[Jt->b[1]].tag : -1;
    }
    /* JinvM = J invM (:505-541) */
    for (int k = 0; k < nj; ++k)
      for (int half = 0; half < 2; ++half) {
        const int bt = jb[2 * k + half];
        if (bt < 0) continue;
        const real im = W->body[bidx[bt]].invMass;
        const real* iI = invI + 12 * bt;
        for (int r = 0; r < ji[k].m; ++r) {
          const real* s = J + (size_t)(ofs[k] + r) * 12 + 6 * half;
          real* t = JinvM + (size_t)(ofs[k] + r) * 12 + 6 * half;
          for (int q = 0; q < 3; ++q) t[q] = s[q] * im;
          for (int q = 0; q < 3; ++q) t[3 + q] = s[3] * iI[q] + s[4] * iI[4 + q] + s[5] * iI[8 + q];
        }
      }
#define DOT6(u, v) ((u)[0] * (v)[0] + (u)[1] * (v)[1] + (u)[2] * (v)[2] + (u)[3] * (v)[3] + (u)[4] * (v)[4] + \
                    (u)[5] * (v)[5])
    /* off-diagonal blocks through shared bodies (:547-607), body 1 then 2 */
    for (int k = 0; k < nj; ++k)
      for (int half = 0; half < 2; ++half) {
        const int bt = jb[2 * k + half];
        if (bt < 0) continue;
        for (int k0 = 0; k0 < k; ++k0) {
          int oh = -1;
          if (jb[2 * k0] == bt) oh = 0;
          else if (jb[2 * k0 + 1] == bt) oh = 1;
          if (oh < 0) continue;
          for (int r = 0; r < ji[k].m; ++r) {
            const real* u = JinvM + (size_t)(ofs[k] + r) * 12 + 6 * half;
            real* Arow = A + (size_t)(ofs[k] + r) * m + ofs[k0];
            for (int c = 0; c < ji[k0].m; ++c) {
              const real* v = J + (size_t)(ofs[k0] + c) * 12 + 6 * oh;
              Arow[c] += DOT6(u, v);
            }
          }
        }
      }
    /* diagonal blocks (:610-627) and cfm / h on the diagonal (:630-637) */
    for (int k = 0; k < nj; ++k)
      for (int r = 0; r < ji[k].m; ++r) {
        real* Arow = A + (size_t)(ofs[k] + r) * m + ofs[k];
        const real* u1 = JinvM + (size_t)(ofs[k] + r) * 12;
        for (int c = 0; c < ji[k].m; ++c) {
          const real* v1 = J + (size_t)(ofs[k] + c) * 12;
          Arow[c] = DOT6(u1, v1);
          if (jb[2 * k + 1] >= 0) Arow[c] += DOT6(u1 + 6, v1 + 6);
        }
      }
    for (int i = 0; i < m; ++i) A[(size_t)i * m + i] += cfm[i] * h1;
    /* rhs = c / h - J (v / h + invM fe) (:643-687) */
    {
      real* tmp1 = (real*)malloc((size_t)nb * 6 * sizeof(real));
      for (int i = 0; i < nb; i++) {
        OBody* b = &W->body[bidx[i]];
        real* t = tmp1 + 6 * i;
        for (int j = 0; j < 3; j++) t[j] = b->facc[j] * b->invMass + b->lvel[j] * h1;
        mul0_331(t + 3, invI + 12 * i, b->tacc);
        for (int q = 0; q < 3; q++) t[3 + q] += b->avel[q] * h1;
      }
      for (int i = 0; i < m; ++i) rhs[i] = rhs[i] * h1;
      for (int k = 0; k < nj; ++k)
        for (int half = 0; half < 2; ++half) {
          const int bt = jb[2 * k + half];
          if (bt < 0) continue;
          for (int r = 0; r < ji[k].m; ++r) {
            const real* u = J + (size_t)(ofs[k] + r) * 12 + 6 * half;
            rhs[ofs[k] + r] -= DOT6(u, tmp1 + 6 * bt);
          }
        }
      free(tmp1);
    }
    real* lambda = (real*)malloc(m * sizeof(real));
    g_lcp_errors += solve_lcp(m, A, lambda, rhs, nub, lo, hi, findex);
    /* cforce = J^T lambda (:720-786), with joint feedback */
    for (int k = 0; k < nj; ++k) {
      OJoint* Jt = &W->joint[ji[k].j];
      for (int half = 0; half < 2; ++half) {
        const int bt = jb[2 * k + half];
        if (bt < 0) continue;
        real s[6] = {0, 0, 0, 0, 0, 0};
        for (int r = 0; r < ji[k].m; ++r) {
          const real* u = J + (size_t)(ofs[k] + r) * 12 + 6 * half;
          const real l = lambda[ofs[k] + r];
          for (int q = 0; q < 6; ++q) s[q] += u[q] * l;
        }
        real* cf = cforce + 6 * bt;
        for (int q = 0; q < 6; ++q) cf[q] += s[q];
        if (Jt->type != ODEGPU_JOINT_CONTACT)
          for (int q = 0; q < 6; ++q) Jt->fb[6 * half + q] = s[q];
      }
    }
#undef DOT6
    free(lo); free(hi); free(J); free(JinvM); free(findex); free(A); free(rhs); free(cfm); free(jb); free(lambda);
  }
  /* velocity update (:790-806), position update, accumulators cleared */
  for (int i = 0; i < nb; i++) {
    OBody* b = &W->body[bidx[i]];
    const real* cf = cforce + 6 * i;
    const real hm = h * b->invMass;
    for (int j = 0; j < 3; j++) b->lvel[j] += (cf[j] + b->facc[j]) * hm;
    real data[3], t3[3];
    for (int k = 0; k < 3; k++) data[k] = (cf[3 + k] + b->tacc[k]) * h;
    mul0_331(t3, invI + 12 * i, data);
    for (int k = 0; k < 3; k++) b->avel[k] += t3[k];
  }
  for (int i = 0; i < nb; i++) step_body(&W->body[bidx[i]], h);
  for (int i = 0; i < nb; i++) {
    OBody* b = &W->body[bidx[i]];
    b->facc[0] = b->facc[1] = b->facc[2] = 0;
    b->tacc[0] = b->tacc[1] = b->tacc[2] = 0;
  }
  free(ji); free(ofs); free(cforce); free(invI);
}

/* ------------------------------------------------------------------------ */
/* world construction from a scene, mirroring the harness's API sequence    */

static void world_init(OWorld* W, const odegpuScene* sc, int w) {
  memset(W, 0, sizeof(*W));
  const odegpuWorldParams* P = &sc->world[w];
  W->sc = sc; W->w = w;
  const int b0 = sc->body_off[w], g0 = sc->geom_off[w], j0 = sc->joint_off[w];
  W->nb = sc->body_off[w + 1] - b0;
  W->ng = sc->geom_off[w + 1] - g0;
  W->nj_persist = sc->joint_off[w + 1] - j0;
  for (int d = 0; d < 3; ++d) W->gravity[d] = P->gravity[d];
  W->erp = P->erp; W->cfm = P->cfm; W->iterations = P->iterations; W->sor_w = P->sor_w;
  W->max_vel = P->max_vel; W->min_depth = P->min_depth; W->dt = P->dt;
  W->max_contacts = P->max_contacts;
  W->body = (OBody*)calloc(W->nb > 0 ? W->nb : 1, sizeof(OBody));
  for (int i = 0; i < W->nb; ++i) {
    OBody* b = &W->body[i];
    const int g = b0 + i;
    for (int k = 0; k < 3; ++k) b->pos[k] = sc->body_pos[3 * g + k];
    for (int k = 0; k < 4; ++k) b->q[k] = sc->body_q[4 * g + k];
    normalize4(b->q);                     /* dBodySetQuaternion, ode.cpp:383-391 */
    r_from_q(b->R, b->q);
    for (int k = 0; k < 3; ++k) b->lvel[k] = sc->body_lvel[3 * g + k];
    for (int k = 0; k < 3; ++k) b->avel[k] = sc->body_avel[3 * g + k];
    const double* I = sc->body_I + 9 * g;
    b->mass = sc->body_mass[g];
    /* dMassSetParameters layout (ode/src/mass.cpp:94-117) */
    memset(b->I, 0, sizeof(b->I));
    b->I[0] = I[0]; b->I[5] = I[4]; b->I[10] = I[8];
    b->I[1] = I[1]; b->I[2] = I[2]; b->I[6] = I[5];
    b->I[4] = I[1]; b->I[8] = I[2]; b->I[9] = I[5];
    if (!invert_pd3(b->I, b->invI)) {
      memset(b->invI, 0, sizeof(b->invI));
      b->invI[0] = b->invI[5] = b->invI[10] = 1;
    }
    b->invMass = 1.0 / b->mass;
    b->flags = sc->body_flags[g];
  }
  W->geom = (OGeom*)calloc(W->ng > 0 ? W->ng : 1, sizeof(OGeom));
  for (int i = 0; i < W->ng; ++i) {
    OGeom* G = &W->geom[i];
    const int g = g0 + i;
    G->type = sc->geom_type[g];
    G->body = sc->geom_body[g];
    G->surface = sc->geom_surface[g];
    for (int k = 0; k < 4; ++k) G->p[k] = sc->geom_param[ODEGPU_GEOM_NPARAM * g + k];
    if (G->type == ODEGPU_GEOM_PLANE) {
      /* make_sure_plane_normal_has_unit_length, ode/src/plane.cpp:40-56 */
      real l = G->p[0] * G->p[0] + G->p[1] * G->p[1] + G->p[2] * G->p[2];
      if (l > 0) {
        l = 1.0 / sqrt(l);
        G->p[0] *= l; G->p[1] *= l; G->p[2] *= l; G->p[3] *= l;
      } else {
        G->p[0] = 1; G->p[1] = 0; G->p[2] = 0; G->p[3] = 0;
      }
    }
    if (G->type == ODEGPU_GEOM_HEIGHTFIELD) {
      G->hf = &sc->heightfields[(int)G->p[0]];
      for (int k = 0; k < 3; ++k) G->hpos[k] = G->hf->pos[k];
      for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) G->hR[r * 4 + c] = G->hf->R[r * 3 + c];
        G->hR[r * 4 + 3] = 0;
      }
    } else {
      memset(G->hR, 0, sizeof(G->hR));
      G->hR[0] = G->hR[5] = G->hR[10] = 1;
    }
  }
  W->cap_j = W->nj_persist + 64;
  W->joint = (OJoint*)calloc(W->cap_j, sizeof(OJoint));
  W->nj = 0;
  for (int i = 0; i < W->nj_persist; ++i) {
    const int g = j0 + i;
    OJoint* J = &W->joint[W->nj];
    const int jj = W->nj++;
    J->type = sc->joint_type[g];
    J->b[0] = J->b[1] = -1;
    const double* a = sc->joint_anchor + 3 * g;
    const double* x1 = sc->joint_axis1 + 3 * g;
    const double* x2 = sc->joint_axis2 + 3 * g;
    const double* jp = sc->joint_param + ODEGPU_JOINT_NPARAM * g;
    const int jb1 = sc->joint_body[2 * g], jb2 = sc->joint_body[2 * g + 1];
    switch (J->type) {
      case ODEGPU_JOINT_BALL:
        J->erp = W->erp; J->cfm = W->cfm;
        joint_attach(W, jj, jb1, jb2);
        set_anchors(W, J, a[0], a[1], a[2], J->anchor1, J->anchor2);
        J->erp = jp[0]; J->cfm = jp[1];
        break;
      case ODEGPU_JOINT_HINGE:
        J->axis1[0] = 1; J->axis2[0] = 1;
        limot_init(&J->lm1, W);
        joint_attach(W, jj, jb1, jb2);
        set_anchors(W, J, a[0], a[1], a[2], J->anchor1, J->anchor2);
        hinge_qrel(W, J);
        set_axes(W, J, x1[0], x1[1], x1[2], J->axis1, J->axis2);
        hinge_qrel(W, J);
        limot_set_all(&J->lm1, jp);
        break;
      case ODEGPU_JOINT_HINGE2: {
        J->axis1[0] = 1; J->axis2[1] = 1;
        J->v1[0] = 1; J->v2[1] = 1;
        limot_init(&J->lm1, W);
        limot_init(&J->lm2, W);
        J->susp_erp = W->erp; J->susp_cfm = W->cfm;
        joint_attach(W, jj, jb1, jb2);
        /* setRelativeValues at attach (ode/src/joints/hinge2.cpp:425-448) */
        {
          real an[3], ax[3], ax1[4], ax2[4], axc[3];
          get_anchor(W, J, an, J->anchor1);
          set_anchors(W, J, an[0], an[1], an[2], J->anchor1, J->anchor2);
          mul0_331(ax, W->body[J->b[0]].R, J->axis1);
          set_axes(W, J, ax[0], ax[1], ax[2], J->axis1, 0);
          if (J->b[1] >= 0) {
            mul0_331(ax, W->body[J->b[1]].R, J->axis2);
            set_axes(W, J, ax[0], ax[1], ax[2], 0, J->axis2);
          }
          hinge2_axis_info(W, J, ax1, ax2, axc, &J->s0, &J->c0);
          hinge2_make_v(W, J);
        }
        set_anchors(W, J, a[0], a[1], a[2], J->anchor1, J->anchor2);
        hinge2_make_v(W, J);
        {
          real ax1[4], ax2[4], axc[3];
          set_axes(W, J, x1[0], x1[1], x1[2], J->axis1, 0);
          hinge2_axis_info(W, J, ax1, ax2, axc, &J->s0, &J->c0);
          hinge2_make_v(W, J);
          set_axes(W, J, x2[0], x2[1], x2[2], 0, J->axis2);
          hinge2_axis_info(W, J, ax1, ax2, axc, &J->s0, &J->c0);
          hinge2_make_v(W, J);
        }
        limot_set_all(&J->lm1, jp);
        limot_set_all(&J->lm2, jp + 9);
        J->susp_erp = jp[18];
        J->susp_cfm = jp[19];
        break;
      }
      case ODEGPU_JOINT_SLIDER:
        /* dJointCreateSlider, dJointAttach (setRelativeValues, overwritten
         * next), dJointSetSliderAxis (ode/src/joints/slider.cpp:250-258) */
        J->axis1[0] = 1;
        limot_init(&J->lm1, W);
        joint_attach(W, jj, jb1, jb2);
        set_axes(W, J, x1[0], x1[1], x1[2], J->axis1, 0);
        slider_offset(W, J);
        hinge_qrel(W, J);
        limot_set_all(&J->lm1, jp);
        break;
      case ODEGPU_JOINT_UNIVERSAL:
        /* dJointCreateUniversal, dJointAttach (setRelativeValues, overwritten
         * next), dJointSetUniversalAnchor / Axis1 / Axis2
         * (ode/src/joints/universal.cpp:396-490); on a reversed joint the
         * API's axis 1 is the second body axis and the other way round */
        J->axis1[0] = 1; J->axis2[1] = 1;
        limot_init(&J->lm1, W);
        limot_init(&J->lm2, W);
        joint_attach(W, jj, jb1, jb2);
        set_anchors(W, J, a[0], a[1], a[2], J->anchor1, J->anchor2);
        universal_qrels(W, J);
        if (J->reverse) set_axes(W, J, x1[0], x1[1], x1[2], 0, J->axis2);
        else set_axes(W, J, x1[0], x1[1], x1[2], J->axis1, 0);
        universal_qrels(W, J);
        if (J->reverse) set_axes(W, J, x2[0], x2[1], x2[2], J->axis1, 0);
        else set_axes(W, J, x2[0], x2[1], x2[2], 0, J->axis2);
        universal_qrels(W, J);
        limot_set_all(&J->lm1, jp);
        limot_set_all(&J->lm2, jp + 9);
        break;
      case ODEGPU_JOINT_AMOTOR: {
        /* dJointCreateAMotor, dJointAttach, dJointSetAMotorMode / NumAxes /
         * Axis (user mode: axes 0..num-1; Euler mode: 0 and 2) / Param / Angle */
        limot_init(&J->lm1, W);
        limot_init(&J->lm2, W);
        limot_init(&J->lm3, W);
        joint_attach(W, jj, jb1, jb2);
        if (J->b[0] >= 0) {
          const int mode = (int)jp[1];
          amotor_set_mode(W, J, mode);
          amotor_set_num(J, (int)jp[0]);
          const double* ax[3] = {a, x1, x2};
          for (int i = 0; i < 3; ++i)
            if (mode == 1 ? i != 1 : i < J->am_num) amotor_set_axis(W, J, i, (int)jp[2 + i], ax[i][0], ax[i][1], ax[i][2]);
          limot_set_all(&J->lm1, jp + 5);
          limot_set_all(&J->lm2, jp + 14);
          limot_set_all(&J->lm3, jp + 23);
          if (mode == 0)
            for (int i = 0; i < J->am_num; ++i) J->am_angle[i] = jp[32 + i];
        }
        break;
      }
      case ODEGPU_JOINT_FIXED:
        /* dJointCreateFixed, dJointAttach, dJointSetFixed, dJointSetFixedParam */
        J->erp = W->erp; J->cfm = W->cfm;
        joint_attach(W, jj, jb1, jb2);
        fixed_set(W, J);
        J->erp = jp[0]; J->cfm = jp[1];
        break;
      default: break;
    }
  }
  for (int i = 0; i < W->nb; ++i) W->body[i].jl_persist = W->body[i].jl_n;
}

static void world_free(OWorld* W) {
  for (int i = 0; i < W->nb; ++i) free(W->body[i].jl);
  free(W->body); free(W->geom); free(W->joint);
}

static int new_contact_joint(OWorld* W) {
  if (W->nj == W->cap_j) {
    W->cap_j *= 2;
    W->joint = (OJoint*)realloc(W->joint, W->cap_j * sizeof(OJoint));
  }
  OJoint* J = &W->joint[W->nj];
  memset(J, 0, sizeof(*J));
  J->type = ODEGPU_JOINT_CONTACT;
  J->b[0] = J->b[1] = -1;
  return W->nj++;
}

/* BuildIslandsAndEstimateStepperMemoryRequirements, ode/src/util.cpp:384-521,
 * followed by dxProcessIslands, :534-568. Bodies are visited newest first
 * (world list order) and each body's joints newest first (attach order
 * reversed); the DFS stack is LIFO. */
static void process_islands(OWorld* W) {
  const int nb = W->nb, nj = W->nj;
  int* ibody = (int*)malloc((size_t)(nb > 0 ? nb : 1) * sizeof(int));
  int* ijoint = (int*)malloc((size_t)(nj > 0 ? nj : 1) * sizeof(int));
  int* stack = (int*)malloc((size_t)(nb > 0 ? nb : 1) * sizeof(int));
  for (int i = 0; i < nb; ++i) W->body[i].tag = 0;
  for (int j = 0; j < nj; ++j) W->joint[j].tag = 0;
  W->last_rows = W->last_islands = 0;
  int island = 0;
  for (int bb = nb - 1; bb >= 0; --bb) {
    if (W->body[bb].tag) continue;
    W->body[bb].tag = 1;
    int nbi = 0, nji = 0, ss = 0;
    ibody[nbi++] = bb;
    int b = bb;
    for (;;) {
      OBody* B = &W->body[b];
      for (int k = B->jl_n - 1; k >= 0; --k) {
        const int j = B->jl[k];
        OJoint* J = &W->joint[j];
        if (J->tag) continue;
        /* dxJoint::isEnabled, ode/src/joints/joint.cpp:66-71 */
        int enabled = (W->body[J->b[0]].invMass > 0) || (J->b[1] >= 0 && W->body[J->b[1]].invMass > 0);
        if (enabled) {
          J->tag = 1;
          ijoint[nji++] = j;
          const int other = (J->b[0] == b) ? J->b[1] : J->b[0];
          if (other >= 0 && W->body[other].tag <= 0) {
            W->body[other].tag = 1;
            stack[ss++] = other;
          }
        } else {
          J->tag = -1;
        }
      }
      if (ss == 0) break;
      b = stack[--ss];
      ibody[nbi++] = b;
    }
    if (g_exact_stepper) exact_stepper(W, ibody, nbi, ijoint, nji, W->dt);
    else quick_stepper(W, ibody, nbi, ijoint, nji, W->dt, island);
    ++island;
  }
  free(ibody); free(ijoint); free(stack);
}

/* dAreConnectedExcluding(b1, b2, dJointTypeContact), ode/src/ode.cpp:1529-1537:
 * contacts are never attached while this is asked, so only persistent joints
 * (the first jl_persist entries of a body's list) can connect. */
static int bodies_jointed(const OWorld* W, int b1, int b2) {
  const OBody* B = &W->body[b1];
  for (int k = 0; k < B->jl_persist; ++k) {
    const OJoint* J = &W->joint[B->jl[k]];
    const int other = (J->b[0] == b1) ? J->b[1] : J->b[0];
    if (other == b2) return 1;
  }
  return 0;
}

/* Bounding radius of a geom on a body (sphere r, box half diagonal, capsule
 * r + length / 2); static geoms have none. */
static real geom_bound(const OGeom* G) {
  switch (G->type) {
    case ODEGPU_GEOM_SPHERE: return G->p[0];
    case ODEGPU_GEOM_BOX: return 0.5 * sqrt(G->p[0] * G->p[0] + G->p[1] * G->p[1] + G->p[2] * G->p[2]);
    case ODEGPU_GEOM_CAPSULE: return G->p[0] + 0.5 * G->p[1];
    case ODEGPU_GEOM_CYLINDER: return sqrt(G->p[0] * G->p[0] + 0.25 * G->p[1] * G->p[1]);
    default: return R_INF;
  }
}

typedef struct { long long key; int g; } CellGeom;
static int cmp_cell(const void* a, const void* b) {
  const long long x = ((const CellGeom*)a)->key, y = ((const CellGeom*)b)->key;
  return (x > y) - (x < y);
}
static int cmp_pair(const void* a, const void* b) {
  const long long x = *(const long long*)a, y = *(const long long*)b;
  return (x > y) - (x < y);
}
static long long cell_key(long long ix, long long iy, long long iz) {
  return ((ix + (1 << 20)) << 42) | ((iy + (1 << 20)) << 21) | (iz + (1 << 20));
}

/* Candidate pairs of a large world in the canonical order, for the CPU
 * baseline: pairs of geoms on bodies within the conservative bounding-sphere
 * test (a uniform grid, cells one test wide), plus every pair of a static and
 * a body geom; sorted by (i, k). Pairs left out cannot produce contacts, so
 * the step is the same as with the full pair loop. Returns the count; *out
 * holds i << 32 | k. */
static int large_world_pairs(OWorld* W, long long** out) {
  const int ng = W->ng;
  real rmax = 0;
  for (int g = 0; g < ng; ++g)
    if (W->geom[g].body >= 0) { const real r = geom_bound(&W->geom[g]); if (r > rmax) rmax = r; }
  const real cell = rmax > 0 ? 1.01 * (2 * rmax * 1.001 + 1e-5) : 1.0;
  CellGeom* cg = (CellGeom*)malloc(sizeof(CellGeom) * (size_t)(ng > 0 ? ng : 1));
  int* cix = (int*)malloc(sizeof(int) * 3 * (size_t)(ng > 0 ? ng : 1));
  int nd = 0;
  for (int g = 0; g < ng; ++g) {
    const int b = W->geom[g].body;
    if (b < 0) continue;
    const real* p = W->body[b].pos;
    const long long ix = (long long)floor(p[0] / cell), iy = (long long)floor(p[1] / cell),
                    iz = (long long)floor(p[2] / cell);
    cix[3 * g] = (int)ix; cix[3 * g + 1] = (int)iy; cix[3 * g + 2] = (int)iz;
    cg[nd].key = cell_key(ix, iy, iz);
    cg[nd].g = g;
    ++nd;
  }
  qsort(cg, nd, sizeof(CellGeom), cmp_cell);
  size_t cap = 1024, n = 0;
  long long* pairs = (long long*)malloc(sizeof(long long) * cap);
#define PUSH_PAIR(a, b)                                                           \
  do {                                                                            \
    if (n == cap) { cap *= 2; pairs = (long long*)realloc(pairs, sizeof(long long) * cap); } \
    pairs[n++] = ((long long)(a) << 32) | (long long)(b);                         \
  } while (0)
  for (int g = 0; g < ng; ++g) {
    const int b = W->geom[g].body;
    if (b < 0) continue;
    for (int s = 0; s < ng; ++s)
      if (W->geom[s].body < 0) { if (s < g) PUSH_PAIR(s, g); else PUSH_PAIR(g, s); }
    const real* p = W->body[b].pos;
    const real rg = geom_bound(&W->geom[g]);
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          const long long key = cell_key(cix[3 * g] + dx, cix[3 * g + 1] + dy, cix[3 * g + 2] + dz);
          int lo = 0, hi = nd;
          while (lo < hi) { const int mid = (lo + hi) / 2; if (cg[mid].key < key) lo = mid + 1; else hi = mid; }
          for (int e = lo; e < nd && cg[e].key == key; ++e) {
            const int k = cg[e].g;
            if (k <= g) continue;
            const int bk = W->geom[k].body;
            if (bk == b) continue;
            const real* q = W->body[bk].pos;
            const real lim = (rg + geom_bound(&W->geom[k])) * 1.001 + 1e-5;
            const real d0 = p[0] - q[0], d1 = p[1] - q[1], d2 = p[2] - q[2];
            if (d0 * d0 + d1 * d1 + d2 * d2 > lim * lim) continue;
            PUSH_PAIR(g, k);
          }
        }
  }
#undef PUSH_PAIR
  qsort(pairs, n, sizeof(long long), cmp_pair);
  free(cg);
  free(cix);
  *out = pairs;
  return (int)n;
}

/* One canonical world step (see include/odegpu_scene.h). */
static int world_step(OWorld* W, int s, double* contacts, int max_rec) {
  const odegpuScene* sc = W->sc;
  int nc = 0;
  OContact cg[16];
  long long* cand = 0;
  const int ncand = W->ng > 512 ? large_world_pairs(W, &cand) : -1;
  const int npair = ncand >= 0 ? ncand : W->ng * (W->ng - 1) / 2;
  for (int pi = 0, i = 0, k = 0; pi < npair; ++pi) {
    if (ncand >= 0) {
      i = (int)(cand[pi] >> 32);
      k = (int)(cand[pi] & 0xffffffff);
    } else {
      /* i < k in order: advance k, then i */
      if (pi == 0) { i = 0; k = 1; }
      else if (++k >= W->ng) { ++i; k = i + 1; }
    }
    {
      const int bi = W->geom[i].body, bk = W->geom[k].body;
      if (bi < 0 && bk < 0) continue;
      if (bi == bk) continue;
      if (bi >= 0 && bk >= 0 && bodies_jointed(W, bi, bk)) continue;
      GeomRef gi, gk;
      fill_ref(W, i, &gi);
      fill_ref(W, k, &gk);
      const int n = do_collide(&gi, &gk, (unsigned)W->max_contacts, cg);
      const int si = W->geom[i].surface, sk = W->geom[k].surface;
      const odegpuSurface* S = &sc->surfaces[si > sk ? si : sk];
      for (int c = 0; c < n; ++c) {
        const int j = new_contact_joint(W);
        OJoint* J = &W->joint[j];
        J->surf = *S;
        for (int q = 0; q < 3; ++q) { J->cpos[q] = cg[c].pos[q]; J->cnormal[q] = cg[c].normal[q]; }
        J->cdepth = cg[c].depth;
        joint_attach(W, j, bi, bk);
        if (contacts && nc < max_rec) {
          double* r = contacts + (size_t)nc * ORACLE_CONTACT_REC;
          for (int q = 0; q < 3; ++q) r[q] = cg[c].pos[q];
          for (int q = 0; q < 3; ++q) r[3 + q] = cg[c].normal[q];
          r[6] = cg[c].depth;
          r[7] = i;
          r[8] = k;
        }
        ++nc;
      }
    }
  }
  free(cand);
  if (sc->n_ctrl_steps > 0) {
    const int cs = s % sc->n_ctrl_steps;
    const int j0 = sc->joint_off[W->w], b0 = sc->body_off[W->w];
    if (sc->joint_stop) {
      /* dJointSet{Hinge,Hinge2,Slider,Universal}Param(dParamLoStop / dParamHiStop): plain
       * assignment (dxJointLimitMotor::set, ode/src/joints/joint.cpp:471-503) */
      for (int i = 0; i < W->nj_persist; ++i) {
        OJoint* J = &W->joint[i];
        if (J->type != ODEGPU_JOINT_HINGE && J->type != ODEGPU_JOINT_HINGE2 &&
            J->type != ODEGPU_JOINT_SLIDER && J->type != ODEGPU_JOINT_UNIVERSAL &&
            J->type != ODEGPU_JOINT_AMOTOR) continue;
        const double v = sc->joint_stop[(size_t)cs * sc->joint_off[sc->n_worlds] + j0 + i];
        const double* jp = sc->joint_param + (size_t)(j0 + i) * ODEGPU_JOINT_NPARAM;
        const double* lp = J->type == ODEGPU_JOINT_AMOTOR ? jp + 5 : jp;
        J->lm1.lostop = isnan(v) ? lp[0] : v;
        J->lm1.histop = isnan(v) ? lp[1] : v;
      }
    }
    if (sc->joint_torque) {
      for (int i = 0; i < W->nj_persist; ++i) {
        const double* t = sc->joint_torque + ((size_t)cs * sc->joint_off[sc->n_worlds] + j0 + i) * 2;
        OJoint* J = &W->joint[i];
        if (J->type == ODEGPU_JOINT_HINGE) {
          /* dJointAddHingeTorque, ode/src/joints/hinge.cpp:326-345 */
          real torque = t[0];
          if (J->reverse) torque = -torque;
          real ax[3];
          if (J->b[0] >= 0) {
            mul0_331(ax, W->body[J->b[0]].R, J->axis1);
            ax[0] *= torque; ax[1] *= torque; ax[2] *= torque;
            OBody* B1 = &W->body[J->b[0]];
            B1->tacc[0] += ax[0]; B1->tacc[1] += ax[1]; B1->tacc[2] += ax[2];
            if (J->b[1] >= 0) {
              OBody* B2 = &W->body[J->b[1]];
              B2->tacc[0] += -ax[0]; B2->tacc[1] += -ax[1]; B2->tacc[2] += -ax[2];
            }
          }
        } else if (J->type == ODEGPU_JOINT_HINGE2) {
          /* dJointAddHinge2Torques, ode/src/joints/hinge2.cpp:393-410 */
          if (J->b[0] >= 0 && J->b[1] >= 0) {
            real a1[3], a2[3];
            mul0_331(a1, W->body[J->b[0]].R, J->axis1);
            mul0_331(a2, W->body[J->b[1]].R, J->axis2);
            a1[0] = a1[0] * t[0] + a2[0] * t[1];
            a1[1] = a1[1] * t[0] + a2[1] * t[1];
            a1[2] = a1[2] * t[0] + a2[2] * t[1];
            OBody* B1 = &W->body[J->b[0]];
            OBody* B2 = &W->body[J->b[1]];
            B1->tacc[0] += a1[0]; B1->tacc[1] += a1[1]; B1->tacc[2] += a1[2];
            B2->tacc[0] += -a1[0]; B2->tacc[1] += -a1[1]; B2->tacc[2] += -a1[2];
          }
        } else if (J->type == ODEGPU_JOINT_SLIDER) {
          /* dJointAddSliderForce, ode/src/joints/slider.cpp:305-342 (a
           * reversed joint computes force -= force, i.e. zero) */
          real force = t[0];
          if (J->reverse) force -= force;
          if (J->b[0] >= 0) {
            OBody* B1 = &W->body[J->b[0]];
            real ax[3];
            mul0_331(ax, B1->R, J->axis1);
            ax[0] *= force; ax[1] *= force; ax[2] *= force;
            B1->facc[0] += ax[0]; B1->facc[1] += ax[1]; B1->facc[2] += ax[2];
            if (J->b[1] >= 0) {
              OBody* B2 = &W->body[J->b[1]];
              B2->facc[0] += -ax[0]; B2->facc[1] += -ax[1]; B2->facc[2] += -ax[2];
              real c[3], ltd[3];
              for (int k = 0; k < 3; ++k) c[k] = 0.5 * (B2->pos[k] - B1->pos[k]);
              cross3(ltd, c, ax);
              for (int k = 0; k < 3; ++k) { B1->tacc[k] += ltd[k]; B2->tacc[k] += ltd[k]; }
            }
          }
        } else if (J->type == ODEGPU_JOINT_AMOTOR) {
          /* dJointAddAMotorTorques(j, t[0], t[1], 0), ode/src/joints/amotor.cpp:474-504 */
          if (J->am_num > 0 && J->b[0] >= 0) {
            real ax[3][4];
            amotor_axes(W, J, ax);
            ax[0][0] *= t[0]; ax[0][1] *= t[0]; ax[0][2] *= t[0];
            if (J->am_num >= 2) {
              for (int k = 0; k < 3; ++k) ax[0][k] += ax[1][k] * t[1];
              if (J->am_num >= 3) for (int k = 0; k < 3; ++k) ax[0][k] += ax[2][k] * 0.0;
            }
            OBody* B1 = &W->body[J->b[0]];
            for (int k = 0; k < 3; ++k) B1->tacc[k] += ax[0][k];
            if (J->b[1] >= 0) {
              OBody* B2 = &W->body[J->b[1]];
              for (int k = 0; k < 3; ++k) B2->tacc[k] += -ax[0][k];
            }
          }
        } else if (J->type == ODEGPU_JOINT_UNIVERSAL) {
          /* dJointAddUniversalTorques, ode/src/joints/universal.cpp:729-754 */
          real t1 = t[0], t2 = t[1];
          if (J->reverse) { real tmp = t1; t1 = -t2; t2 = -tmp; }
          if (J->b[0] >= 0) {
            real a1[3], a2[3];
            universal_axes(W, J, a1, a2);
            for (int k = 0; k < 3; ++k) a1[k] = a1[k] * t1 + a2[k] * t2;
            OBody* B1 = &W->body[J->b[0]];
            B1->tacc[0] += a1[0]; B1->tacc[1] += a1[1]; B1->tacc[2] += a1[2];
            if (J->b[1] >= 0) {
              OBody* B2 = &W->body[J->b[1]];
              B2->tacc[0] += -a1[0]; B2->tacc[1] += -a1[1]; B2->tacc[2] += -a1[2];
            }
          }
        }
      }
    }
    if (sc->body_force) {
      for (int i = 0; i < W->nb; ++i) {
        const double* f = sc->body_force + ((size_t)cs * sc->body_off[sc->n_worlds] + b0 + i) * 6;
        OBody* B = &W->body[i];
        B->facc[0] += f[0]; B->facc[1] += f[1]; B->facc[2] += f[2];
        B->tacc[0] += f[3]; B->tacc[1] += f[4]; B->tacc[2] += f[5];
      }
    }
  }
  process_islands(W);
  /* dJointGroupEmpty, ode/src/ode.cpp:1305-1332: contacts leave every list */
  W->nj = W->nj_persist;
  for (int i = 0; i < W->nb; ++i) W->body[i].jl_n = W->body[i].jl_persist;
  return nc;
}

static void read_state(const OWorld* W, double* out) {
  for (int i = 0; i < W->nb; ++i) {
    const OBody* b = &W->body[i];
    double* r = out + ORACLE_BODY_REC * i;
    for (int k = 0; k < 3; ++k) r[k] = b->pos[k];
    for (int k = 0; k < 4; ++k) r[3 + k] = b->q[k];
    for (int k = 0; k < 3; ++k) r[7 + k] = b->lvel[k];
    for (int k = 0; k < 3; ++k) r[10 + k] = b->avel[k];
  }
}

/* Overwrite every body's state after the world was built from the scene (joint
 * anchors, axes and reference angles stay as the scene set them up). The
 * quaternion is taken as given and R follows from it (dRfromQ), which is how
 * a step treats the state it starts from. */
static void write_state(OWorld* W, const double* in) {
  for (int i = 0; i < W->nb; ++i) {
    OBody* b = &W->body[i];
    const double* r = in + ORACLE_BODY_REC * i;
    for (int k = 0; k < 3; ++k) b->pos[k] = r[k];
    for (int k = 0; k < 4; ++k) b->q[k] = r[3 + k];
    for (int k = 0; k < 3; ++k) b->lvel[k] = r[7 + k];
    for (int k = 0; k < 3; ++k) b->avel[k] = r[10 + k];
    r_from_q(b->R, b->q);
  }
}

int oracle_run_world_from(const odegpuScene* sc, int w, int n_steps, const double* init_state,
                          double* final_state) {
  if (!sc || w < 0 || w >= sc->n_worlds || n_steps < 0 || !init_state) return -1;
  OWorld W;
  world_init(&W, sc, w);
  g_seed = sc->world[w].seed;
  write_state(&W, init_state);
  for (int s = 0; s < n_steps; ++s) world_step(&W, s, 0, 0);
  if (final_state) read_state(&W, final_state);
  world_free(&W);
  return 0;
}

int oracle_run_world(const odegpuScene* sc, int w, int n_steps, double* state, int* ncontacts,
                     double* contacts, int max_rec, double* feedback, unsigned int* seed_out) {
  if (!sc || w < 0 || w >= sc->n_worlds || n_steps < 0) return -1;
  OWorld W;
  world_init(&W, sc, w);
  g_seed = sc->world[w].seed;
  if (state) read_state(&W, state);
  for (int s = 0; s < n_steps; ++s) {
    const int nc = world_step(&W, s, contacts ? contacts + (size_t)s * max_rec * ORACLE_CONTACT_REC : 0,
                              max_rec);
    if (ncontacts) ncontacts[s] = nc;
    if (state) read_state(&W, state + (size_t)(s + 1) * W.nb * ORACLE_BODY_REC);
    if (feedback)
      for (int i = 0; i < W.nj_persist; ++i)
        memcpy(feedback + ((size_t)s * W.nj_persist + i) * 12, W.joint[i].fb, 12 * sizeof(double));
    if (seed_out) seed_out[s] = g_seed;
  }
  world_free(&W);
  return 0;
}

typedef struct {
  const odegpuScene* sc;
  int w_begin, w_end, n_steps, stride, t;
  double* out;
  long long contacts;
} ThreadArg;

static void* run_worlds_thread(void* p) {
  ThreadArg* a = (ThreadArg*)p;
  const odegpuScene* sc = a->sc;
  for (int w = a->w_begin + a->t; w < a->w_end; w += a->stride) {
    OWorld W;
    world_init(&W, sc, w);
    g_seed = sc->world[w].seed;
    for (int s = 0; s < a->n_steps; ++s) a->contacts += world_step(&W, s, 0, 0);
    if (a->out) read_state(&W, a->out + (size_t)(sc->body_off[w] - sc->body_off[a->w_begin]) * ORACLE_BODY_REC);
    world_free(&W);
  }
  return 0;
}

long long oracle_run_worlds(const odegpuScene* sc, int w_begin, int w_end, int n_steps, int n_threads,
                            double* final_state) {
  if (n_threads < 1) n_threads = 1;
  pthread_t* th = (pthread_t*)malloc(n_threads * sizeof(pthread_t));
  ThreadArg* args = (ThreadArg*)calloc(n_threads, sizeof(ThreadArg));
  for (int t = 0; t < n_threads; ++t) {
    args[t].sc = sc; args[t].w_begin = w_begin; args[t].w_end = w_end; args[t].n_steps = n_steps;
    args[t].stride = n_threads; args[t].t = t; args[t].out = final_state;
    pthread_create(&th[t], 0, run_worlds_thread, &args[t]);
  }
  long long total = 0;
  for (int t = 0; t < n_threads; ++t) { pthread_join(th[t], 0); total += args[t].contacts; }
  free(th); free(args);
  return total;
}

typedef struct {
  const odegpuScene* sc;
  int w_begin, w_end, step0, n_steps, t;
  const double* state_in;
  const unsigned* seed_in;
  double* state_out;
  unsigned* seed_out;
  int* counts;
  int* next;          /* shared work counter (worlds are handed out in order) */
  pthread_mutex_t* mu;
} FromArg;

static void* step_from_thread(void* p) {
  FromArg* a = (FromArg*)p;
  const odegpuScene* sc = a->sc;
  const size_t b_first = (size_t)sc->body_off[a->w_begin];
  for (;;) {
    pthread_mutex_lock(a->mu);
    const int w = (*a->next)++;
    pthread_mutex_unlock(a->mu);
    if (w >= a->w_end) break;
    OWorld W;
    world_init(&W, sc, w);
    const size_t b0 = (size_t)sc->body_off[w] - b_first;
    if (a->state_in) write_state(&W, a->state_in + b0 * ORACLE_BODY_REC);
    g_seed = a->seed_in ? a->seed_in[w - a->w_begin] : sc->world[w].seed;
    for (int s = 0; s < a->n_steps; ++s) {
      const int nc = world_step(&W, a->step0 + s, 0, 0);
      if (a->counts) {
        int* c = a->counts + ((size_t)(w - a->w_begin) * a->n_steps + s) * 3;
        c[0] = nc; c[1] = W.last_rows; c[2] = W.last_islands;
      }
    }
    if (a->state_out) read_state(&W, a->state_out + b0 * ORACLE_BODY_REC);
    if (a->seed_out) a->seed_out[w - a->w_begin] = g_seed;
    world_free(&W);
  }
  return 0;
}

int oracle_step_worlds_from(const odegpuScene* sc, int w_begin, int w_end, int step0, int n_steps,
                            int n_threads, const double* state_in, const unsigned int* seed_in,
                            double* state_out, unsigned int* seed_out, int* counts) {
  if (!sc || w_begin < 0 || w_end > sc->n_worlds || w_begin > w_end || n_steps < 0 || step0 < 0) return -1;
  if (n_threads < 1) n_threads = 1;
  pthread_t* th = (pthread_t*)malloc(n_threads * sizeof(pthread_t));
  FromArg* args = (FromArg*)calloc(n_threads, sizeof(FromArg));
  pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
  int next = w_begin;
  for (int t = 0; t < n_threads; ++t) {
    FromArg* a = &args[t];
    a->sc = sc; a->w_begin = w_begin; a->w_end = w_end; a->step0 = step0; a->n_steps = n_steps; a->t = t;
    a->state_in = state_in; a->seed_in = seed_in; a->state_out = state_out; a->seed_out = seed_out;
    a->counts = counts; a->next = &next; a->mu = &mu;
    pthread_create(&th[t], 0, step_from_thread, a);
  }
  for (int t = 0; t < n_threads; ++t) pthread_join(th[t], 0);
  free(th); free(args);
  return 0;
}

int oracle_step_world_contacts(const odegpuScene* sc, int w, int step, const double* state_in,
                               unsigned int seed, double* contacts, int max_rec, double* state_out) {
  if (!sc || w < 0 || w >= sc->n_worlds || step < 0) return -1;
  OWorld W;
  world_init(&W, sc, w);
  if (state_in) write_state(&W, state_in);
  g_seed = seed;
  const int nc = world_step(&W, step, contacts, max_rec);
  if (state_out) read_state(&W, state_out);
  world_free(&W);
  return nc;
}

int oracle_tap_step(const odegpuScene* sc, int w, int pre_steps, oracleTap* tap) {
  if (!sc || !tap || w < 0 || w >= sc->n_worlds) return -1;
  OWorld W;
  world_init(&W, sc, w);
  g_seed = sc->world[w].seed;
  for (int s = 0; s < pre_steps; ++s) world_step(&W, s, 0, 0);
  tap->n_islands = 0;
  tap->seed_before = g_seed;
  W.tap = tap;
  world_step(&W, pre_steps, 0, 0);
  int total = 0;
  for (int i = 0; i < tap->n_islands; ++i) total += tap->island_rows[i];
  world_free(&W);
  return total;
}

int oracle_collide(int t1, const double* p1, const double* pos1, const double* R1, int t2, const double* p2,
                   const double* pos2, const double* R2, int flags, double* out) {
  OGeom G[2];
  real pos[2][3], R[2][12];
  const int tt[2] = {t1, t2};
  const double* pp[2] = {p1, p2};
  const double* ps[2] = {pos1, pos2};
  const double* rs[2] = {R1, R2};
  GeomRef ref[2];
  for (int g = 0; g < 2; ++g) {
    memset(&G[g], 0, sizeof(OGeom));
    G[g].type = tt[g];
    for (int k = 0; k < 4; ++k) G[g].p[k] = pp[g][k];
    if (tt[g] == ODEGPU_GEOM_PLANE) {
      real l = G[g].p[0] * G[g].p[0] + G[g].p[1] * G[g].p[1] + G[g].p[2] * G[g].p[2];
      if (l > 0) {
        l = 1.0 / sqrt(l);
        G[g].p[0] *= l; G[g].p[1] *= l; G[g].p[2] *= l; G[g].p[3] *= l;
      }
      memset(pos[g], 0, sizeof(pos[g]));
      memset(R[g], 0, sizeof(R[g]));
    } else {
      for (int k = 0; k < 3; ++k) pos[g][k] = ps[g][k];
      for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) R[g][r * 4 + c] = rs[g][r * 3 + c];
        R[g][r * 4 + 3] = 0;
      }
    }
    ref[g].type = tt[g]; ref[g].pos = pos[g]; ref[g].R = R[g]; ref[g].p = G[g].p; ref[g].g = &G[g];
  }
  OContact c[16];
  int n = do_collide(&ref[0], &ref[1], (unsigned)flags, c);
  for (int i = 0; i < n; ++i) {
    double* r = out + 9 * i;
    for (int q = 0; q < 3; ++q) r[q] = c[i].pos[q];
    for (int q = 0; q < 3; ++q) r[3 + q] = c[i].normal[q];
    r[6] = c[i].depth; r[7] = 0; r[8] = 0;
  }
  return n;
}

int oracle_collide_hf(const odegpuHeightfield* H, int t2, const double* p2, const double* pos2, const double* R2,
                      int flags, double* out) {
  OGeom G[2];
  real R[2][12], pos[2][3];
  memset(G, 0, sizeof(G));
  G[0].type = ODEGPU_GEOM_HEIGHTFIELD;
  G[0].hf = H;
  G[1].type = t2;
  for (int k = 0; k < 4; ++k) G[1].p[k] = p2[k];
  for (int k = 0; k < 3; ++k) { pos[0][k] = H->pos[k]; pos[1][k] = pos2[k]; }
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) { R[0][r * 4 + c] = H->R[r * 3 + c]; R[1][r * 4 + c] = R2[r * 3 + c]; }
    R[0][r * 4 + 3] = R[1][r * 4 + 3] = 0;
  }
  GeomRef a = {ODEGPU_GEOM_HEIGHTFIELD, pos[0], R[0], G[0].p, &G[0]};
  GeomRef b = {t2, pos[1], R[1], G[1].p, &G[1]};
  OContact c[64];
  if ((flags & 0xffff) > 64) flags = (flags & ~0xffff) | 64;
  const int n = do_collide(&a, &b, (unsigned)flags, c);
  for (int i = 0; i < n; ++i) {
    double* r = out + 9 * i;
    for (int q = 0; q < 3; ++q) r[q] = c[i].pos[q];
    for (int q = 0; q < 3; ++q) r[3 + q] = c[i].normal[q];
    r[6] = c[i].depth; r[7] = 0; r[8] = 0;
  }
  return n;
}
