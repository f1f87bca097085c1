// collide.cuh -- FP32 primitive narrowphase on the device.
//
// Each collider keeps the case structure of its reference counterpart (cited
// per function) so that the number of contacts, their order and which feature
// produced them match the reference on the same inputs; only the arithmetic
// precision differs (FP32 here, FP64 in the oracle).
#pragma once
#include "dmath.cuh"

namespace og {

struct Contact {
  float pos[3], normal[3], depth;
};

// Placement + class parameters of one geom as the colliders see it.
struct GeomView {
  int type;
  float pos[3];
  float R[12];
  float p[4];   // sphere r / box sides / capsule, cylinder r,len / plane a,b,c,d / ray length
};

enum { G_SPHERE = 0, G_BOX = 1, G_CAPSULE = 2, G_CYLINDER = 3, G_PLANE = 4, G_RAY = 5, G_HEIGHTFIELD = 9 };
constexpr unsigned kContactsUnimportant = 0x80000000u;

// dCollideSpheres (ode/src/collision_util.cpp:38-67)
OG_HD int collide_spheres(const float* p1, float r1, const float* p2, float r2, Contact* c) {
  float t[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
  float d = sqrtf(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
  if (d > (r1 + r2)) return 0;
  if (d <= 0.f) {
    c->pos[0] = p1[0]; c->pos[1] = p1[1]; c->pos[2] = p1[2];
    c->normal[0] = 1.f; c->normal[1] = 0.f; c->normal[2] = 0.f;
    c->depth = r1 + r2;
  } else {
    float d1 = 1.0f / d;
    c->normal[0] = (p1[0] - p2[0]) * d1;
    c->normal[1] = (p1[1] - p2[1]) * d1;
    c->normal[2] = (p1[2] - p2[2]) * d1;
    float k = 0.5f * (r2 - r1 - d);
    c->pos[0] = p1[0] + c->normal[0] * k;
    c->pos[1] = p1[1] + c->normal[1] * k;
    c->pos[2] = p1[2] + c->normal[2] * k;
    c->depth = r1 + r2 - d;
  }
  return 1;
}

// dCollideSphereBox (ode/src/sphere.cpp:131-219)
OG_HD int collide_sphere_box(const GeomView& s, const GeomView& b, Contact* c) {
  float l[3], t[4], p[3], q[3], r[3];
  int onborder = 0;
  const float* R = b.R;
  p[0] = s.pos[0] - b.pos[0];
  p[1] = s.pos[1] - b.pos[1];
  p[2] = s.pos[2] - b.pos[2];
  for (int i = 0; i < 3; ++i) {
    l[i] = b.p[i] * 0.5f;
    t[i] = dot3s(p, R + i, 1, 4);
    if (t[i] < -l[i]) { t[i] = -l[i]; onborder = 1; }
    if (t[i] > l[i]) { t[i] = l[i]; onborder = 1; }
  }
  if (!onborder) {
    float min_distance = l[0] - fabsf(t[0]);
    int mini = 0;
    for (int i = 1; i < 3; i++) {
      float fd = l[i] - fabsf(t[i]);
      if (fd < min_distance) { min_distance = fd; mini = i; }
    }
    c->pos[0] = s.pos[0]; c->pos[1] = s.pos[1]; c->pos[2] = s.pos[2];
    float tmp[3] = {0.f, 0.f, 0.f};
    tmp[mini] = (t[mini] > 0.f) ? 1.0f : -1.0f;
    mul0_331(c->normal, R, tmp);
    c->depth = min_distance + s.p[0];
    return 1;
  }
  t[3] = 0.f;
  mul0_331(q, R, t);
  r[0] = p[0] - q[0]; r[1] = p[1] - q[1]; r[2] = p[2] - q[2];
  float depth = s.p[0] - sqrtf(dot3(r, r));
  if (depth < 0.f) return 0;
  c->pos[0] = q[0] + b.pos[0];
  c->pos[1] = q[1] + b.pos[1];
  c->pos[2] = q[2] + b.pos[2];
  c->normal[0] = r[0]; c->normal[1] = r[1]; c->normal[2] = r[2];
  safe_normalize3(c->normal);
  c->depth = depth;
  return 1;
}

// dCollideSpherePlane (ode/src/sphere.cpp:222-251)
OG_HD int collide_sphere_plane(const GeomView& s, const GeomView& pl, Contact* c) {
  const float* P = pl.p;
  float k = dot3(s.pos, P);
  float depth = P[3] - k + s.p[0];
  if (depth >= 0.f) {
    c->normal[0] = P[0]; c->normal[1] = P[1]; c->normal[2] = P[2];
    c->pos[0] = s.pos[0] - P[0] * s.p[0];
    c->pos[1] = s.pos[1] - P[1] * s.p[0];
    c->pos[2] = s.pos[2] - P[2] * s.p[0];
    c->depth = depth;
    return 1;
  }
  return 0;
}

// dLineClosestApproach (ode/src/collision_util.cpp:70-92)
OG_HD void line_closest_approach(const float* pa, const float* ua, const float* pb, const float* ub,
                                 float* alpha, float* beta) {
  float p[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
  float uaub = dot3(ua, ub);
  float q1 = dot3(ua, p);
  float q2 = -dot3(ub, p);
  float d = 1.f - uaub * uaub;
  if (d <= 0.0001f) { *alpha = 0.f; *beta = 0.f; }
  else {
    d = 1.0f / d;
    *alpha = (q1 + uaub * q2) * d;
    *beta = (uaub * q1 + q2) * d;
  }
}

// intersectRectQuad (ode/src/box.cpp:187-245): clip the quad p against the
// rectangle |x| < h[0], |y| < h[1]; emits points in the reference's order.
OG_HD int intersect_rect_quad(const float h[2], float p[8], float ret[16]) {
  int nq = 4, nr = 0;
  float buffer[16];
  float* q = p;
  float* r = ret;
  for (int dir = 0; dir <= 1; dir++) {
    for (int sign = -1; sign <= 1; sign += 2) {
      float* pq = q;
      float* pr = r;
      nr = 0;
      for (int i = nq; i > 0; i--) {
        if (sign * pq[dir] < h[dir]) {
          pr[0] = pq[0]; pr[1] = pq[1];
          pr += 2; nr++;
          if (nr & 8) { q = r; goto done; }
        }
        float* nextq = (i > 1) ? pq + 2 : q;
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
  if (q != ret)
    for (int i = 0; i < nr * 2; ++i) ret[i] = q[i];
  return nr;
}

// cullPoints (ode/src/box.cpp:249-322)
OG_HD void cull_points(int n, const float p[], int m, int i0, int iret[]) {
  int i, j;
  float a, cx, cy, q;
  if (n == 1) { cx = p[0]; cy = p[1]; }
  else if (n == 2) { cx = 0.5f * (p[0] + p[2]); cy = 0.5f * (p[1] + p[3]); }
  else {
    a = 0.f; cx = 0.f; cy = 0.f;
    for (i = 0; i < (n - 1); i++) {
      q = p[i * 2] * p[i * 2 + 3] - p[i * 2 + 2] * p[i * 2 + 1];
      a += q;
      cx += q * (p[i * 2] + p[i * 2 + 2]);
      cy += q * (p[i * 2 + 1] + p[i * 2 + 3]);
    }
    q = p[n * 2 - 2] * p[1] - p[0] * p[n * 2 - 1];
    a = 1.0f / (3.0f * (a + q));
    cx = a * (cx + q * (p[n * 2 - 2] + p[0]));
    cy = a * (cy + q * (p[n * 2 - 1] + p[1]));
  }
  float A[8];
  for (i = 0; i < n; i++) A[i] = atan2f(p[i * 2 + 1] - cy, p[i * 2] - cx);
  int avail[8];
  for (i = 0; i < n; i++) avail[i] = 1;
  avail[i0] = 0;
  iret[0] = i0;
  int k = 1;
  // The reference mixes a double-precision pi into these FP32 expressions
  // (M_PI is double in <math.h>); the same promotions are kept here.
  const double kPiD = 3.14159265358979323846;
  for (j = 1; j < m; j++) {
    a = (float)((double)j * (2.0 * kPiD / m) + (double)A[i0]);
    if ((double)a > kPiD) a -= (float)(2.0 * kPiD);
    float maxdiff = 1e9f, diff;
    int best = i0;
    for (i = 0; i < n; i++) {
      if (avail[i]) {
        diff = fabsf(A[i] - a);
        if ((double)diff > kPiD) diff = (float)(2.0 * kPiD - (double)diff);
        if (diff < maxdiff) { maxdiff = diff; best = i; }
      }
    }
    iret[k] = best;
    avail[best] = 0;
    k++;
  }
}

// dBoxBox (ode/src/box.cpp:331-713): separating-axis test over 15 axes (1.05
// fudge on the edge axes), then edge-edge or face clipping + culling.
// depth_out / code_out (for the ODE API's dBoxBox): the deepest penetration
// once the normal is known, and the contact's code on the paths that make
// contacts, as box.cpp:461, :501, :710 set them.
OG_HD int box_box(const float* p1, const float* R1, const float* side1, const float* p2,
                  const float* R2, const float* side2, float* normal, unsigned flags,
                  Contact* contact, float* depth_out = nullptr, int* code_out = nullptr) {
  const float fudge_factor = 1.05f;
  float p[3], pp[3], normalC[3] = {0.f, 0.f, 0.f};
  const float* normalR = nullptr;
  float A[3], B[3], s, s2, l, e1;
  int invert_normal, code;
  p[0] = p2[0] - p1[0]; p[1] = p2[1] - p1[1]; p[2] = p2[2] - p1[2];
  mul1_331(pp, R1, p);
  A[0] = side1[0] * 0.5f; A[1] = side1[1] * 0.5f; A[2] = side1[2] * 0.5f;
  B[0] = side2[0] * 0.5f; B[1] = side2[1] * 0.5f; B[2] = side2[2] * 0.5f;
  const float R11 = dot3s(R1 + 0, R2 + 0, 4, 4), R12 = dot3s(R1 + 0, R2 + 1, 4, 4), R13 = dot3s(R1 + 0, R2 + 2, 4, 4);
  const float R21 = dot3s(R1 + 1, R2 + 0, 4, 4), R22 = dot3s(R1 + 1, R2 + 1, 4, 4), R23 = dot3s(R1 + 1, R2 + 2, 4, 4);
  const float R31 = dot3s(R1 + 2, R2 + 0, 4, 4), R32 = dot3s(R1 + 2, R2 + 1, 4, 4), R33 = dot3s(R1 + 2, R2 + 2, 4, 4);
  const float Q11 = fabsf(R11), Q12 = fabsf(R12), Q13 = fabsf(R13);
  const float Q21 = fabsf(R21), Q22 = fabsf(R22), Q23 = fabsf(R23);
  const float Q31 = fabsf(R31), Q32 = fabsf(R32), Q33 = fabsf(R33);
  s = -INFINITY;
  invert_normal = 0;
  code = 0;
  do {
#define OG_TST_FACE(expr1, expr2, norm, cc)                          \
  e1 = (expr1);                                                      \
  s2 = fabsf(e1) - (expr2);                                          \
  if (s2 > 0.f) return 0;                                            \
  if (s2 > s) {                                                      \
    s = s2; normalR = norm; invert_normal = (e1 < 0.f); code = (cc); \
    if (flags & kContactsUnimportant) break;                         \
  }
    OG_TST_FACE(pp[0], (A[0] + B[0] * Q11 + B[1] * Q12 + B[2] * Q13), R1 + 0, 1);
    OG_TST_FACE(pp[1], (A[1] + B[0] * Q21 + B[1] * Q22 + B[2] * Q23), R1 + 1, 2);
    OG_TST_FACE(pp[2], (A[2] + B[0] * Q31 + B[1] * Q32 + B[2] * Q33), R1 + 2, 3);
    OG_TST_FACE(dot3s(R2 + 0, p, 4, 1), (A[0] * Q11 + A[1] * Q21 + A[2] * Q31 + B[0]), R2 + 0, 4);
    OG_TST_FACE(dot3s(R2 + 1, p, 4, 1), (A[0] * Q12 + A[1] * Q22 + A[2] * Q32 + B[1]), R2 + 1, 5);
    OG_TST_FACE(dot3s(R2 + 2, p, 4, 1), (A[0] * Q13 + A[1] * Q23 + A[2] * Q33 + B[2]), R2 + 2, 6);
#undef OG_TST_FACE
#define OG_TST_EDGE(expr1, expr2, n1, n2, n3, cc)                        \
  e1 = (expr1);                                                          \
  s2 = fabsf(e1) - (expr2);                                              \
  if (s2 > 0.f) return 0;                                                \
  l = sqrtf((n1) * (n1) + (n2) * (n2) + (n3) * (n3));                    \
  if (l > 0.f) {                                                         \
    s2 /= l;                                                             \
    if (s2 * fudge_factor > s) {                                         \
      s = s2; normalR = nullptr;                                         \
      normalC[0] = (n1) / l; normalC[1] = (n2) / l; normalC[2] = (n3) / l; \
      invert_normal = (e1 < 0.f); code = (cc);                           \
      if (flags & kContactsUnimportant) break;                           \
    }                                                                    \
  }
    OG_TST_EDGE(pp[2] * R21 - pp[1] * R31, (A[1] * Q31 + A[2] * Q21 + B[1] * Q13 + B[2] * Q12), 0.f, -R31, R21, 7);
    OG_TST_EDGE(pp[2] * R22 - pp[1] * R32, (A[1] * Q32 + A[2] * Q22 + B[0] * Q13 + B[2] * Q11), 0.f, -R32, R22, 8);
    OG_TST_EDGE(pp[2] * R23 - pp[1] * R33, (A[1] * Q33 + A[2] * Q23 + B[0] * Q12 + B[1] * Q11), 0.f, -R33, R23, 9);
    OG_TST_EDGE(pp[0] * R31 - pp[2] * R11, (A[0] * Q31 + A[2] * Q11 + B[1] * Q23 + B[2] * Q22), R31, 0.f, -R11, 10);
    OG_TST_EDGE(pp[0] * R32 - pp[2] * R12, (A[0] * Q32 + A[2] * Q12 + B[0] * Q23 + B[2] * Q21), R32, 0.f, -R12, 11);
    OG_TST_EDGE(pp[0] * R33 - pp[2] * R13, (A[0] * Q33 + A[2] * Q13 + B[0] * Q22 + B[1] * Q21), R33, 0.f, -R13, 12);
    OG_TST_EDGE(pp[1] * R11 - pp[0] * R21, (A[0] * Q21 + A[1] * Q11 + B[1] * Q33 + B[2] * Q32), -R21, R11, 0.f, 13);
    OG_TST_EDGE(pp[1] * R12 - pp[0] * R22, (A[0] * Q22 + A[1] * Q12 + B[0] * Q33 + B[2] * Q31), -R22, R12, 0.f, 14);
    OG_TST_EDGE(pp[1] * R13 - pp[0] * R23, (A[0] * Q23 + A[1] * Q13 + B[0] * Q32 + B[1] * Q31), -R23, R13, 0.f, 15);
#undef OG_TST_EDGE
  } while (0);
  if (!code) return 0;
  if (normalR) {
    normal[0] = normalR[0]; normal[1] = normalR[4]; normal[2] = normalR[8];
  } else {
    mul0_331(normal, R1, normalC);
  }
  if (invert_normal) { normal[0] = -normal[0]; normal[1] = -normal[1]; normal[2] = -normal[2]; }
  if (depth_out) *depth_out = -s;
  const float depth = -s;
  int i, j;
  if (code > 6) {
    float pa[3], pb[3], sign, alpha, beta, ua[3], ub[3];
    for (i = 0; i < 3; i++) pa[i] = p1[i];
    for (j = 0; j < 3; j++) {
      sign = (dot3s(normal, R1 + j, 1, 4) > 0.f) ? 1.0f : -1.0f;
      for (i = 0; i < 3; i++) pa[i] += sign * A[j] * R1[i * 4 + j];
    }
    for (i = 0; i < 3; i++) pb[i] = p2[i];
    for (j = 0; j < 3; j++) {
      sign = (dot3s(normal, R2 + j, 1, 4) > 0.f) ? -1.0f : 1.0f;
      for (i = 0; i < 3; i++) pb[i] += sign * B[j] * R2[i * 4 + j];
    }
    for (i = 0; i < 3; i++) ua[i] = R1[((code)-7) / 3 + i * 4];
    for (i = 0; i < 3; i++) ub[i] = R2[((code)-7) % 3 + i * 4];
    line_closest_approach(pa, ua, pb, ub, &alpha, &beta);
    for (i = 0; i < 3; i++) pa[i] += ua[i] * alpha;
    for (i = 0; i < 3; i++) pb[i] += ub[i] * beta;
    for (i = 0; i < 3; i++) contact[0].pos[i] = 0.5f * (pa[i] + pb[i]);
    contact[0].depth = depth;
    if (code_out) *code_out = code;
    return 1;
  }
  const float *Ra, *Rb, *pa, *pb, *Sa, *Sb;
  if (code <= 3) { Ra = R1; Rb = R2; pa = p1; pb = p2; Sa = A; Sb = B; }
  else { Ra = R2; Rb = R1; pa = p2; pb = p1; Sa = B; Sb = A; }
  float normal2[3], nr[3], anr[3];
  if (code <= 3) { normal2[0] = normal[0]; normal2[1] = normal[1]; normal2[2] = normal[2]; }
  else { normal2[0] = -normal[0]; normal2[1] = -normal[1]; normal2[2] = -normal[2]; }
  mul1_331(nr, Rb, normal2);
  anr[0] = fabsf(nr[0]); anr[1] = fabsf(nr[1]); anr[2] = fabsf(nr[2]);
  int lanr, a1, a2;
  if (anr[1] > anr[0]) {
    if (anr[1] > anr[2]) { a1 = 0; lanr = 1; a2 = 2; }
    else { a1 = 0; a2 = 1; lanr = 2; }
  } else {
    if (anr[0] > anr[2]) { lanr = 0; a1 = 1; a2 = 2; }
    else { a1 = 0; a2 = 1; lanr = 2; }
  }
  float center[3];
  if (nr[lanr] < 0.f) {
    for (i = 0; i < 3; i++) center[i] = pb[i] - pa[i] + Sb[lanr] * Rb[i * 4 + lanr];
  } else {
    for (i = 0; i < 3; i++) center[i] = pb[i] - pa[i] - Sb[lanr] * Rb[i * 4 + lanr];
  }
  int codeN, code1, code2;
  codeN = (code <= 3) ? code - 1 : code - 4;
  if (codeN == 0) { code1 = 1; code2 = 2; }
  else if (codeN == 1) { code1 = 0; code2 = 2; }
  else { code1 = 0; code2 = 1; }
  float quad[8];
  const float c1 = dot3s(center, Ra + code1, 1, 4);
  const float c2 = dot3s(center, Ra + code2, 1, 4);
  float m11 = dot3s(Ra + code1, Rb + a1, 4, 4);
  float m12 = dot3s(Ra + code1, Rb + a2, 4, 4);
  float m21 = dot3s(Ra + code2, Rb + a1, 4, 4);
  float m22 = dot3s(Ra + code2, Rb + a2, 4, 4);
  {
    float k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
    quad[0] = c1 - k1 - k3; quad[1] = c2 - k2 - k4;
    quad[2] = c1 - k1 + k3; quad[3] = c2 - k2 + k4;
    quad[4] = c1 + k1 + k3; quad[5] = c2 + k2 + k4;
    quad[6] = c1 + k1 - k3; quad[7] = c2 + k2 - k4;
  }
  const float rect[2] = {Sa[code1], Sa[code2]};
  float ret[16];
  const int n = intersect_rect_quad(rect, quad, ret);
  if (n < 1) return 0;
  float point[3 * 8], dep[8];
  const float det1 = 1.0f / (m11 * m22 - m12 * m21);
  m11 *= det1; m12 *= det1; m21 *= det1; m22 *= det1;
  int cnum = 0;
  for (j = 0; j < n; j++) {
    float k1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
    float k2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
    for (i = 0; i < 3; i++) point[cnum * 3 + i] = center[i] + k1 * Rb[i * 4 + a1] + k2 * Rb[i * 4 + a2];
    dep[cnum] = Sa[codeN] - dot3(normal2, point + cnum * 3);
    if (dep[cnum] >= 0.f) {
      ret[cnum * 2] = ret[j * 2];
      ret[cnum * 2 + 1] = ret[j * 2 + 1];
      cnum++;
      if ((cnum | kContactsUnimportant) == (flags & (0xffffu | kContactsUnimportant))) break;
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
    float maxdepth = dep[0];
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
  if (code_out) *code_out = code;
  return cnum;
}

// dCollideBoxBox (ode/src/box.cpp:716-742): normal returned negated.
OG_HD int collide_box_box(const GeomView& a, const GeomView& b, unsigned flags, Contact* c) {
  float normal[3];
  const int num = box_box(a.pos, a.R, a.p, b.pos, b.R, b.p, normal, flags, c);
  for (int i = 0; i < num; i++) {
    c[i].normal[0] = -normal[0]; c[i].normal[1] = -normal[1]; c[i].normal[2] = -normal[2];
  }
  return num;
}

// dCollideBoxPlane (ode/src/box.cpp:745-878): deepest vertex, then vertices
// along the two sides with the smallest projections, the fourth by vector sum.
OG_HD int collide_box_plane(const GeomView& bx, const GeomView& pl, unsigned flags, Contact* c) {
  const float* R = bx.R;
  const float* n = pl.p;
  const float* side = bx.p;
  const float Aa[3] = {side[0] * dot3s(n, R + 0, 1, 4), side[1] * dot3s(n, R + 1, 1, 4),
                       side[2] * dot3s(n, R + 2, 1, 4)};
  const float Bb[3] = {fabsf(Aa[0]), fabsf(Aa[1]), fabsf(Aa[2])};
  const float depth = n[3] + 0.5f * (Bb[0] + Bb[1] + Bb[2]) - dot3(n, bx.pos);
  if (depth < 0.f) return 0;
  int maxc = flags & 0xffff;
  if (maxc > 4) maxc = 4;
  float p[3] = {bx.pos[0], bx.pos[1], bx.pos[2]};
  for (int i = 0; i < 3; ++i) {
    const float sgn = (Aa[i] > 0.f) ? -0.5f : 0.5f;
    p[0] += sgn * side[i] * R[0 + i];
    p[1] += sgn * side[i] * R[4 + i];
    p[2] += sgn * side[i] * R[8 + i];
  }
  c[0].pos[0] = p[0]; c[0].pos[1] = p[1]; c[0].pos[2] = p[2];
  c[0].depth = depth;
  int ret = 1;
  if (maxc > 1) {
    // sequence of sides to walk, as chosen by the reference's branch ladder
    int s1, s2;
    if (Bb[0] < Bb[1]) {
      if (Bb[2] < Bb[0]) { s1 = 2; s2 = (Bb[0] < Bb[1]) ? 0 : 1; }
      else { s1 = 0; s2 = (Bb[1] < Bb[2]) ? 1 : 2; }
    } else {
      if (Bb[2] < Bb[1]) { s1 = 2; s2 = (Bb[0] < Bb[1]) ? 0 : 1; }
      else { s1 = 1; s2 = (Bb[0] < Bb[2]) ? 0 : 2; }
    }
    const int seq[2] = {s1, s2};
    for (int k = 0; k < 2 && k + 1 < maxc; ++k) {
      const int sd = seq[k];
      if (depth - Bb[sd] < 0.f) break;
      const float sg = (Aa[sd] > 0.f) ? 1.f : -1.f;
      c[k + 1].pos[0] = p[0] + sg * side[sd] * R[0 + sd];
      c[k + 1].pos[1] = p[1] + sg * side[sd] * R[4 + sd];
      c[k + 1].pos[2] = p[2] + sg * side[sd] * R[8 + sd];
      c[k + 1].depth = depth - Bb[sd];
      ret++;
    }
  }
  if (maxc == 4 && ret == 3) {
    const float d4 = c[1].depth + c[2].depth - depth;
    if (d4 > 0.f) {
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

// dCollideCapsulePlane (ode/src/capsule.cpp:352-411)
OG_HD int collide_capsule_plane(const GeomView& cp, const GeomView& pl, unsigned flags, Contact* c) {
  const float* R = cp.R;
  const float* P = pl.p;
  const float radius = cp.p[0], lz = cp.p[1];
  const float sign = (dot3s(P, R + 2, 1, 4) > 0.f) ? -1.0f : 1.0f;
  float p[3];
  p[0] = cp.pos[0] + R[2] * lz * 0.5f * sign;
  p[1] = cp.pos[1] + R[6] * lz * 0.5f * sign;
  p[2] = cp.pos[2] + R[10] * lz * 0.5f * sign;
  float k = dot3(p, P);
  float depth = P[3] - k + radius;
  if (depth < 0.f) return 0;
  c[0].normal[0] = P[0]; c[0].normal[1] = P[1]; c[0].normal[2] = P[2];
  c[0].pos[0] = p[0] - P[0] * radius;
  c[0].pos[1] = p[1] - P[1] * radius;
  c[0].pos[2] = p[2] - P[2] * radius;
  c[0].depth = depth;
  int nc = 1;
  if ((flags & 0xffff) >= 2) {
    p[0] = cp.pos[0] - R[2] * lz * 0.5f * sign;
    p[1] = cp.pos[1] - R[6] * lz * 0.5f * sign;
    p[2] = cp.pos[2] - R[10] * lz * 0.5f * sign;
    k = dot3(p, P);
    depth = P[3] - k + radius;
    if (depth >= 0.f) {
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

// dCollideCapsuleSphere (ode/src/capsule.cpp:130-160)
OG_HD int collide_capsule_sphere(const GeomView& cp, const GeomView& sp, Contact* c) {
  const float* R = cp.R;
  float alpha = R[2] * (sp.pos[0] - cp.pos[0]) + R[6] * (sp.pos[1] - cp.pos[1]) + R[10] * (sp.pos[2] - cp.pos[2]);
  const float lz2 = cp.p[1] * 0.5f;
  if (alpha > lz2) alpha = lz2;
  if (alpha < -lz2) alpha = -lz2;
  const float p[3] = {cp.pos[0] + alpha * R[2], cp.pos[1] + alpha * R[6], cp.pos[2] + alpha * R[10]};
  return collide_spheres(p, cp.p[0], sp.pos, sp.p[0], c);
}

// dCollideSpheresZeroDist (ode/src/capsule.cpp:164-176)
OG_HD int collide_spheres_zero_dist(const float* p1, float r1, float r2, const float* normal, Contact* c) {
  c->normal[0] = normal[0]; c->normal[1] = normal[1]; c->normal[2] = normal[2];
  c->depth = r1 + r2;
  const float k = 0.5f * (r2 - r1);
  c->pos[0] = p1[0] + c->normal[0] * k;
  c->pos[1] = p1[1] + c->normal[1] * k;
  c->pos[2] = p1[2] + c->normal[2] * k;
  return 1;
}

// dClosestLineBoxPoints (ode/src/collision_util.cpp:247-372), dSINGLE epsilon:
// t walks along the segment p1 -> p2 through the box's clip planes until
// d|D(t)|^2/dt turns non-negative.
OG_HD void closest_line_box_points(const float* p1, const float* p2, const float* c, const float* R,
                                   const float* side, float* lret, float* bret) {
  float tmp[3], s[3], v[3], sign[3], v2[3], h[3], tanchor[3];
  int region[3];
  tmp[0] = p1[0] - c[0]; tmp[1] = p1[1] - c[1]; tmp[2] = p1[2] - c[2];
  mul1_331(s, R, tmp);
  tmp[0] = p2[0] - p1[0]; tmp[1] = p2[1] - p1[1]; tmp[2] = p2[2] - p1[2];
  mul1_331(v, R, tmp);
  for (int i = 0; i < 3; i++) {
    if (v[i] < 0.f) { s[i] = -s[i]; v[i] = -v[i]; sign[i] = -1.f; }
    else sign[i] = 1.f;
  }
  for (int i = 0; i < 3; i++) v2[i] = v[i] * v[i];
  for (int i = 0; i < 3; i++) h[i] = 0.5f * side[i];
  const float tanchor_eps = 1e-19f;
  for (int i = 0; i < 3; i++) {
    if (v[i] > tanchor_eps) {
      if (s[i] < -h[i]) { region[i] = -1; tanchor[i] = (-h[i] - s[i]) / v[i]; }
      else { region[i] = (s[i] > h[i]); tanchor[i] = (h[i] - s[i]) / v[i]; }
    } else {
      region[i] = 0;
      tanchor[i] = 2.f;
    }
  }
  float t = 0.f, dd2dt = 0.f;
  for (int i = 0; i < 3; i++) dd2dt -= (region[i] ? v2[i] : 0.f) * tanchor[i];
  if (dd2dt < 0.f) {
    bool done = false;
    do {
      float next_t = 1.f;
      for (int i = 0; i < 3; i++)
        if (tanchor[i] > t && tanchor[i] < 1.f && tanchor[i] < next_t) next_t = tanchor[i];
      float next_dd2dt = 0.f;
      for (int i = 0; i < 3; i++) next_dd2dt += (region[i] ? v2[i] : 0.f) * (next_t - tanchor[i]);
      if (next_dd2dt >= 0.f) {
        const float m = (next_dd2dt - dd2dt) / (next_t - t);
        t -= dd2dt / m;
        done = true;
        break;
      }
      for (int i = 0; i < 3; i++) {
        if (tanchor[i] == next_t) {
          tanchor[i] = (h[i] - s[i]) / v[i];
          region[i]++;
        }
      }
      t = next_t;
      dd2dt = next_dd2dt;
    } while (t < 1.f);
    if (!done) t = 1.f;
  }
  for (int i = 0; i < 3; i++) lret[i] = p1[i] + t * tmp[i];
  for (int i = 0; i < 3; i++) {
    tmp[i] = sign[i] * (s[i] + t * v[i]);
    if (tmp[i] < -h[i]) tmp[i] = -h[i];
    else if (tmp[i] > h[i]) tmp[i] = h[i];
  }
  mul0_331(s, R, tmp);
  for (int i = 0; i < 3; i++) bret[i] = s[i] + c[i];
}

// dClosestLineSegmentPoints (ode/src/collision_util.cpp:109-209): vertex-vertex,
// then edge-vertex, then edge-edge features.
OG_HD void closest_segment_points(const float* a1, const float* a2, const float* b1, const float* b2, float* cp1,
                                  float* cp2) {
  float a1a2[3], b1b2[3], a1b1[3], a1b2[3], a2b1[3], a2b2[3], n[3];
  for (int i = 0; i < 3; ++i) { a1a2[i] = a2[i] - a1[i]; b1b2[i] = b2[i] - b1[i]; a1b1[i] = b1[i] - a1[i]; }
  const float da1 = dot3(a1a2, a1b1), db1 = dot3(b1b2, a1b1);
  if (da1 <= 0.f && db1 >= 0.f) { for (int i = 0; i < 3; ++i) { cp1[i] = a1[i]; cp2[i] = b1[i]; } return; }
  for (int i = 0; i < 3; ++i) a1b2[i] = b2[i] - a1[i];
  const float da2 = dot3(a1a2, a1b2), db2 = dot3(b1b2, a1b2);
  if (da2 <= 0.f && db2 <= 0.f) { for (int i = 0; i < 3; ++i) { cp1[i] = a1[i]; cp2[i] = b2[i]; } return; }
  for (int i = 0; i < 3; ++i) a2b1[i] = b1[i] - a2[i];
  const float da3 = dot3(a1a2, a2b1), db3 = dot3(b1b2, a2b1);
  if (da3 >= 0.f && db3 >= 0.f) { for (int i = 0; i < 3; ++i) { cp1[i] = a2[i]; cp2[i] = b1[i]; } return; }
  for (int i = 0; i < 3; ++i) a2b2[i] = b2[i] - a2[i];
  const float da4 = dot3(a1a2, a2b2), db4 = dot3(b1b2, a2b2);
  if (da4 >= 0.f && db4 <= 0.f) { for (int i = 0; i < 3; ++i) { cp1[i] = a2[i]; cp2[i] = b2[i]; } return; }
  const float la = dot3(a1a2, a1a2);
  if (da1 >= 0.f && da3 <= 0.f) {
    const float k = da1 / la;
    for (int i = 0; i < 3; ++i) n[i] = a1b1[i] - k * a1a2[i];
    if (dot3(b1b2, n) >= 0.f) {
      for (int i = 0; i < 3; ++i) { cp1[i] = a1[i] + k * a1a2[i]; cp2[i] = b1[i]; }
      return;
    }
  }
  if (da2 >= 0.f && da4 <= 0.f) {
    const float k = da2 / la;
    for (int i = 0; i < 3; ++i) n[i] = a1b2[i] - k * a1a2[i];
    if (dot3(b1b2, n) <= 0.f) {
      for (int i = 0; i < 3; ++i) { cp1[i] = a1[i] + k * a1a2[i]; cp2[i] = b2[i]; }
      return;
    }
  }
  const float lb = dot3(b1b2, b1b2);
  if (db1 <= 0.f && db2 >= 0.f) {
    const float k = -db1 / lb;
    for (int i = 0; i < 3; ++i) n[i] = -a1b1[i] - k * b1b2[i];
    if (dot3(a1a2, n) >= 0.f) {
      for (int i = 0; i < 3; ++i) { cp1[i] = a1[i]; cp2[i] = b1[i] + k * b1b2[i]; }
      return;
    }
  }
  if (db3 <= 0.f && db4 >= 0.f) {
    const float k = -db3 / lb;
    for (int i = 0; i < 3; ++i) n[i] = -a2b1[i] - k * b1b2[i];
    if (dot3(a1a2, n) <= 0.f) {
      for (int i = 0; i < 3; ++i) { cp1[i] = a2[i]; cp2[i] = b1[i] + k * b1b2[i]; }
      return;
    }
  }
  const float k = dot3(a1a2, b1b2);
  float det = la * lb - k * k;
  if (det <= 0.f) { for (int i = 0; i < 3; ++i) { cp1[i] = a1[i]; cp2[i] = b1[i]; } return; }
  det = 1.0f / det;
  const float alpha = (lb * da1 - k * db1) * det;
  const float beta = (k * da1 - la * db1) * det;
  for (int i = 0; i < 3; ++i) { cp1[i] = a1[i] + alpha * a1a2[i]; cp2[i] = b1[i] + beta * b1b2[i]; }
}

// dCollideCapsuleBox (ode/src/capsule.cpp:178-229), dSINGLE minimum distance
OG_HD int collide_capsule_box(const GeomView& cp, const GeomView& bx, Contact* c) {
  const float clen = cp.p[1] * 0.5f;
  float p1[3], p2[3], pl[3], pb[3];
  for (int i = 0; i < 3; ++i) {
    p1[i] = cp.pos[i] + clen * cp.R[4 * i + 2];
    p2[i] = cp.pos[i] - clen * cp.R[4 * i + 2];
  }
  closest_line_box_points(p1, p2, bx.pos, bx.R, bx.p, pl, pb);
  const float dx = pl[0] - pb[0], dy = pl[1] - pb[1], dz = pl[2] - pb[2];
  if (sqrtf(dx * dx + dy * dy + dz * dz) < 1e-9f) {
    float normal[3] = {pb[0] - bx.pos[0], pb[1] - bx.pos[1], pb[2] - bx.pos[2]};
    safe_normalize3(normal);
    return collide_spheres_zero_dist(pl, cp.p[0], 0.f, normal, c);
  }
  return collide_spheres(pl, cp.p[0], pb, 0.f, c);
}

// dCollideCapsuleCapsule (ode/src/capsule.cpp:232-350): near-parallel axes
// give up to two contacts along the overlap, otherwise the closest points of
// the two segments.
OG_HD int collide_capsule_capsule(const GeomView& g1, const GeomView& g2, unsigned flags, Contact* c) {
  const float tolerance = 1e-5f;
  const float lz1 = g1.p[1] * 0.5f, lz2 = g2.p[1] * 0.5f;
  const float* pos1 = g1.pos;
  const float* pos2 = g2.pos;
  const float axis1[3] = {g1.R[2], g1.R[6], g1.R[10]};
  float axis2[3] = {g2.R[2], g2.R[6], g2.R[10]};
  float sphere1[3], sphere2[3];
  const float a1a2 = dot3(axis1, axis2);
  const float det = 1.0f - a1a2 * a1a2;
  if (det < tolerance) {
    if (a1a2 < 0.f) { axis2[0] = -axis2[0]; axis2[1] = -axis2[1]; axis2[2] = -axis2[2]; }
    float q[3];
    for (int i = 0; i < 3; i++) q[i] = pos1[i] - pos2[i];
    const float k = dot3(axis1, q);
    const float a1lo = -lz1, a1hi = lz1, a2lo = -lz2 - k, a2hi = lz2 - k;
    const float lo = (a1lo > a2lo) ? a1lo : a2lo;
    const float hi = (a1hi < a2hi) ? a1hi : a2hi;
    if (lo <= hi) {
      const int num_contacts = (int)(flags & 0xffff);
      if (num_contacts >= 2 && lo < hi) {
        for (int i = 0; i < 3; i++) sphere1[i] = pos1[i] + lo * axis1[i];
        for (int i = 0; i < 3; i++) sphere2[i] = pos2[i] + (lo + k) * axis2[i];
        const int n1 = collide_spheres(sphere1, g1.p[0], sphere2, g2.p[0], c);
        if (n1) {
          for (int i = 0; i < 3; i++) sphere1[i] = pos1[i] + hi * axis1[i];
          for (int i = 0; i < 3; i++) sphere2[i] = pos2[i] + (hi + k) * axis2[i];
          const int n2 = collide_spheres(sphere1, g1.p[0], sphere2, g2.p[0], c + 1);
          if (n2) return 2;
        }
      }
      const float alpha1 = (lo + hi) * 0.5f;
      const float alpha2 = alpha1 + k;
      for (int i = 0; i < 3; i++) sphere1[i] = pos1[i] + alpha1 * axis1[i];
      for (int i = 0; i < 3; i++) sphere2[i] = pos2[i] + alpha2 * axis2[i];
      return collide_spheres(sphere1, g1.p[0], sphere2, g2.p[0], c);
    }
  }
  float a1[3], a2[3], b1[3], b2[3];
  for (int i = 0; i < 3; ++i) {
    a1[i] = pos1[i] + axis1[i] * lz1;
    a2[i] = pos1[i] - axis1[i] * lz1;
    b1[i] = pos2[i] + axis2[i] * lz2;
    b2[i] = pos2[i] - axis2[i] * lz2;
  }
  closest_segment_points(a1, a2, b1, b2, sphere1, sphere2);
  return collide_spheres(sphere1, g1.p[0], sphere2, g2.p[0], c);
}

// ---- rays (ode/src/ray.cpp). A ray geom holds its length in p[0], starts at
// pos and points along column 2 of R. Each collider returns at most one
// contact; its depth is the distance from the start along the ray.

// ray_sphere_helper (ray.cpp:196-233); mode 1 takes the exit point.
OG_HD int ray_sphere_helper(const GeomView& ray, const float* spos, float radius, Contact* c, int mode) {
  const float* rp = ray.pos;
  const float* R = ray.R;
  const float q[3] = {rp[0] - spos[0], rp[1] - spos[1], rp[2] - spos[2]};
  const float B = q[0] * R[2] + q[1] * R[6] + q[2] * R[10];
  const float C = dot3(q, q) - radius * radius;
  float k = B * B - C;
  if (k < 0.f) return 0;
  k = sqrtf(k);
  float alpha;
  if (mode && C >= 0.f) {
    alpha = -B + k;
    if (alpha < 0.f) return 0;
  } else {
    alpha = -B - k;
    if (alpha < 0.f) {
      alpha = -B + k;
      if (alpha < 0.f) return 0;
    }
  }
  if (alpha > ray.p[0]) return 0;
  for (int i = 0; i < 3; ++i) c->pos[i] = rp[i] + alpha * R[i * 4 + 2];
  const float nsign = (C < 0.f || mode) ? -1.f : 1.f;
  for (int i = 0; i < 3; ++i) c->normal[i] = nsign * (c->pos[i] - spos[i]);
  safe_normalize3(c->normal);
  c->depth = alpha;
  return 1;
}

// dCollideRayBox (ray.cpp:253-350): slab test in the box frame, the ray
// mirrored so that its direction has no negative component.
OG_HD int collide_ray_box(const GeomView& ray, const GeomView& bx, Contact* c) {
  const float* rp = ray.pos;
  const float* RR = ray.R;
  const float* BR = bx.R;
  float tmp[3] = {rp[0] - bx.pos[0], rp[1] - bx.pos[1], rp[2] - bx.pos[2]};
  float s[3], v[3], sign[3];
  mul1_331(s, BR, tmp);
  tmp[0] = RR[2]; tmp[1] = RR[6]; tmp[2] = RR[10];
  mul1_331(v, BR, tmp);
  for (int i = 0; i < 3; ++i) {
    if (v[i] < 0.f) { s[i] = -s[i]; v[i] = -v[i]; sign[i] = 1.f; }
    else sign[i] = -1.f;
  }
  const float h[3] = {0.5f * bx.p[0], 0.5f * bx.p[1], 0.5f * bx.p[2]};
  if ((s[0] < -h[0] && v[0] <= 0.f) || s[0] > h[0] || (s[1] < -h[1] && v[1] <= 0.f) || s[1] > h[1] ||
      (s[2] < -h[2] && v[2] <= 0.f) || s[2] > h[2] || (v[0] == 0.f && v[1] == 0.f && v[2] == 0.f))
    return 0;
  float lo = -INFINITY, hi = INFINITY;
  int nlo = 0, nhi = 0;
  for (int i = 0; i < 3; ++i) {
    if (v[i] != 0.f) {
      float k = (-h[i] - s[i]) / v[i];
      if (k > lo) { lo = k; nlo = i; }
      k = (h[i] - s[i]) / v[i];
      if (k < hi) { hi = k; nhi = i; }
    }
  }
  if (lo > hi) return 0;
  const bool front = lo >= 0.f;
  const float alpha = front ? lo : hi;
  const int n = front ? nlo : nhi;
  if (alpha < 0.f || alpha > ray.p[0]) return 0;
  for (int i = 0; i < 3; ++i) {
    c->pos[i] = rp[i] + alpha * RR[i * 4 + 2];
    c->normal[i] = BR[i * 4 + n] * sign[n];
  }
  c->depth = alpha;
  return 1;
}

// dCollideRayCapsule (ray.cpp:352-465): the infinite cylinder first, then the
// cap sphere on the side where the hit (or the start) lies.
OG_HD int collide_ray_capsule(const GeomView& ray, const GeomView& cp, Contact* c) {
  const float* rp = ray.pos;
  const float* RR = ray.R;
  const float* CR = cp.R;
  const float* cpos = cp.pos;
  const float radius = cp.p[0];
  const float lz2 = cp.p[1] * 0.5f;
  const float cs[3] = {rp[0] - cpos[0], rp[1] - cpos[1], rp[2] - cpos[2]};
  float k = CR[2] * cs[0] + CR[6] * cs[1] + CR[10] * cs[2];
  float q[3], r[3];
  for (int i = 0; i < 3; ++i) q[i] = k * CR[i * 4 + 2] - cs[i];
  const float C = dot3(q, q) - radius * radius;
  int inside = 0;
  if (C < 0.f) {
    if (k < -lz2) k = -lz2;
    else if (k > lz2) k = lz2;
    for (int i = 0; i < 3; ++i) r[i] = cpos[i] + k * CR[i * 4 + 2];
    if ((rp[0] - r[0]) * (rp[0] - r[0]) + (rp[1] - r[1]) * (rp[1] - r[1]) + (rp[2] - r[2]) * (rp[2] - r[2]) <
        radius * radius)
      inside = 1;
  }
  if (!inside && C < 0.f) {
    k = (k < 0.f) ? -lz2 : lz2;
  } else {
    const float uv = CR[2] * RR[2] + CR[6] * RR[6] + CR[10] * RR[10];
    for (int i = 0; i < 3; ++i) r[i] = uv * CR[i * 4 + 2] - RR[i * 4 + 2];
    float A = dot3(r, r);
    const float B = 2.f * dot3(q, r);
    k = B * B - 4.f * A * C;
    if (k < 0.f) {
      if (!inside) return 0;
      k = (uv < 0.f) ? -lz2 : lz2;
    } else {
      k = sqrtf(k);
      A = 1.0f / (2.f * A);
      float alpha = (-B - k) * A;
      if (alpha < 0.f) {
        alpha = (-B + k) * A;
        if (alpha < 0.f) return 0;
      }
      if (alpha > ray.p[0]) return 0;
      for (int i = 0; i < 3; ++i) c->pos[i] = rp[i] + alpha * RR[i * 4 + 2];
      for (int i = 0; i < 3; ++i) q[i] = c->pos[i] - cpos[i];
      k = q[0] * CR[2] + q[1] * CR[6] + q[2] * CR[10];
      const float nsign = inside ? -1.f : 1.f;
      if (k >= -lz2 && k <= lz2) {
        for (int i = 0; i < 3; ++i) c->normal[i] = nsign * (c->pos[i] - (cpos[i] + k * CR[i * 4 + 2]));
        safe_normalize3(c->normal);
        c->depth = alpha;
        return 1;
      }
      k = (k < 0.f) ? -lz2 : lz2;
    }
  }
  for (int i = 0; i < 3; ++i) q[i] = cpos[i] + k * CR[i * 4 + 2];
  return ray_sphere_helper(ray, q, radius, c, inside);
}

// dCollideRayPlane (ray.cpp:467-498)
OG_HD int collide_ray_plane(const GeomView& ray, const GeomView& pl, Contact* c) {
  const float* rp = ray.pos;
  const float* RR = ray.R;
  const float* P = pl.p;
  float alpha = P[3] - (P[0] * rp[0] + P[1] * rp[1] + P[2] * rp[2]);
  const float nsign = (alpha > 0.f) ? -1.f : 1.f;
  const float k = P[0] * RR[2] + P[1] * RR[6] + P[2] * RR[10];
  if (k == 0.f) return 0;
  alpha /= k;
  if (alpha < 0.f || alpha > ray.p[0]) return 0;
  for (int i = 0; i < 3; ++i) {
    c->pos[i] = rp[i] + alpha * RR[i * 4 + 2];
    c->normal[i] = nsign * P[i];
  }
  c->depth = alpha;
  return 1;
}

// ---- cylinders (flat-ended, ode/src/cylinder.cpp): p[0] radius, p[1] length
// along column 2 of R. kCylTol is the dSINGLE build's "toleranz".
constexpr float kCylTol = 1e-4f;

// dCollideCylinderSphere (ode/src/collision_cylinder_sphere.cpp:56-276): side,
// disc or rim contact from the sphere centre's axial (s) and radial (t)
// distances.
OG_HD int collide_cylinder_sphere(const GeomView& cy, const GeomView& sp, Contact* c) {
  const float radius = cy.p[0], length = cy.p[1];
  const float* cp = cy.pos;
  const float r2 = sp.p[0];
  const float* S = sp.pos;
  const float v[3] = {cy.R[2], cy.R[6], cy.R[10]};
  float s = length * 0.5f;
  float P1[3], P2[3], C[3];
  for (int i = 0; i < 3; ++i) { P2[i] = v[i] * s + cp[i]; P1[i] = v[i] * -s + cp[i]; }
  s = (S[0] - P1[0]) * v[0] - (P1[1] - S[1]) * v[1] - (P1[2] - S[2]) * v[2];
  if (s < (-r2) || s > (length + r2)) return 0;
  for (int i = 0; i < 3; ++i) C[i] = s * v[i] + P1[i] - S[i];
  const float t = sqrtf(dot3(C, C));
  if (t > (radius + r2)) return 0;
  if (t > radius && (s < 0.f || s > length)) {
    const float* P = (s <= 0.f) ? P1 : P2;
    const float ds = (s <= 0.f) ? s : (s - length);
    c->depth = r2 - sqrtf(ds * ds + (t - radius) * (t - radius));
    if (c->depth < 0.f) return 0;
    for (int i = 0; i < 3; ++i) c->pos[i] = C[i] / t * -radius + P[i];
    for (int i = 0; i < 3; ++i) c->normal[i] = (c->pos[i] - S[i]) / (r2 - c->depth);
    return 1;
  } else if ((radius - t) <= s && (radius - t) <= (length - s)) {
    c->depth = (r2 + radius) - t;
    if (c->depth < 0.f) return 0;
    if (t > (r2 + kCylTol)) {
      for (int i = 0; i < 3; ++i) C[i] /= t;
      for (int i = 0; i < 3; ++i) { c->pos[i] = C[i] * r2 + S[i]; c->normal[i] = C[i]; }
    } else {
      for (int i = 0; i < 3; ++i) { c->pos[i] = C[i] + S[i]; c->normal[i] = C[i] / t; }
    }
    return 1;
  }
  if (s <= (length * 0.5f)) {
    c->depth = s + r2;
    if (c->depth < 0.f) return 0;
    for (int i = 0; i < 3; ++i) { c->pos[i] = r2 * v[i] + S[i]; c->normal[i] = v[i]; }
  } else {
    c->depth = (r2 + length - s);
    if (c->depth < 0.f) return 0;
    for (int i = 0; i < 3; ++i) { c->pos[i] = r2 * -v[i] + S[i]; c->normal[i] = -v[i]; }
  }
  return 1;
}

// dCollideCylinderPlane (ode/src/collision_cylinder_plane.cpp:43-265): four rim
// points of the lower disc when the axis is parallel to the plane normal (within
// kCylTol), else the deepest rim point of each disc.
OG_HD int collide_cylinder_plane(const GeomView& cy, const GeomView& pl, unsigned flags, Contact* c) {
  const int maxc = (int)(flags & 0xffff);
  const float radius = cy.p[0], length = cy.p[1];
  const float* cp = cy.pos;
  const float* P = pl.p;
  const float v[3] = {cy.R[2], cy.R[6], cy.R[10]};
  float s = length * 0.5f;
  float P1[3], P2[3];
  for (int i = 0; i < 3; ++i) { P2[i] = v[i] * s + cp[i]; P1[i] = v[i] * -s + cp[i]; }
  int n = 0;
  s = v[0] * P[0] + v[1] * P[1] + v[2] * P[2];
  if (s < 0.f) s += 1.0f;
  else s -= 1.0f;
  if (s < kCylTol && s > (-kCylTol)) {
    float Q[3];
    s = P[3] - dot3(P, P1);
    float t = P[3] - dot3(P, P2);
    if (s >= t) {
      if (s >= 0.f) { Q[0] = P1[0]; Q[1] = P1[1]; Q[2] = P1[2]; }
      else return 0;
    } else {
      if (t >= 0.f) { Q[0] = P2[0]; Q[1] = P2[1]; Q[2] = P2[2]; }
      else return 0;
    }
    float V1[3], V2[3];
    if (v[0] < kCylTol && v[0] > (-kCylTol)) { V1[0] = v[0] + 1.0f; V1[1] = v[1]; V1[2] = v[2]; }
    else { V1[0] = v[0]; V1[1] = v[1] + 1.0f; V1[2] = v[2]; }
    cross3(V2, V1, v);
    t = sqrtf(dot3(V2, V2));
    t = radius / t;
    for (int i = 0; i < 3; ++i) V2[i] *= t;
    cross3(V1, V2, v);
    for (int k = 0; k < 4; ++k) {
      const float* A = (k < 2) ? V1 : V2;
      Contact* o = &c[n];
      for (int i = 0; i < 3; ++i) o->pos[i] = (k & 1) ? Q[i] - A[i] : Q[i] + A[i];
      o->depth = P[3] - dot3(P, o->pos);
      if (o->depth > 0.f) {
        o->normal[0] = P[0]; o->normal[1] = P[1]; o->normal[2] = P[2];
        if (++n >= maxc) return n;
      }
    }
  } else {
    const float t = dot3(P, v);
    float C[3];
    for (int i = 0; i < 3; ++i) C[i] = v[i] * t - P[i];
    s = sqrtf(dot3(C, C));
    s = radius / s;
    for (int i = 0; i < 3; ++i) C[i] *= s;
    Contact* o = &c[n];
    for (int i = 0; i < 3; ++i) o->pos[i] = C[i] + P1[i];
    o->depth = P[3] - dot3(P, o->pos);
    if (o->depth >= 0.f) {
      o->normal[0] = P[0]; o->normal[1] = P[1]; o->normal[2] = P[2];
      if (++n >= maxc) return n;
    }
    o = &c[n];
    for (int i = 0; i < 3; ++i) o->pos[i] = C[i] + P2[i];
    o->depth = P[3] - P[0] * o->pos[0] - P[1] * o->pos[1] - P[2] * o->pos[2];
    if (o->depth >= 0.f) {
      o->normal[0] = P[0]; o->normal[1] = P[1]; o->normal[2] = P[2];
      if (++n >= maxc) return n;
    }
  }
  return n;
}

// dCollideRayCylinder (ode/src/ray.cpp:500-698): the flat caps when the ray
// starts inside the infinite cylinder running along the axis (the test uses
// FLT_EPSILON, dEpsilon of dSINGLE), else the curved side between the caps.
OG_HD int collide_ray_cylinder(const GeomView& ray, const GeomView& cy, Contact* c) {
  const float* RR = ray.R;
  const float* CR = cy.R;
  const float half = cy.p[1] * 0.5f;
  float r[3] = {ray.pos[0] - cy.pos[0], ray.pos[1] - cy.pos[1], ray.pos[2] - cy.pos[2]};
  float d = CR[2] * r[0] + CR[6] * r[1] + CR[10] * r[2];
  float q[3];
  for (int i = 0; i < 3; ++i) q[i] = (d * CR[i * 4 + 2]) - r[i];
  const float C = dot3(q, q) - (cy.p[0] * cy.p[0]);
  const float uv = CR[2] * RR[2] + CR[6] * RR[6] + CR[10] * RR[10];
  for (int i = 0; i < 3; ++i) r[i] = (uv * CR[i * 4 + 2]) - RR[i * 4 + 2];
  float A = dot3(r, r);
  const float B = 2.f * dot3(q, r);
  float k = B * B - 4.f * A * C;
  if (k < 1.1920929e-7f && C <= 0.f) {
    const float uvsign = (uv < 0.f) ? -1.0f : 1.0f;
    const float internal = (d >= -half && d <= +half) ? -1.0f : 1.0f;
    if (((uv > 0.f) && (d + (uvsign * ray.p[0]) < half * internal)) ||
        ((uv < 0.f) && (d + (uvsign * ray.p[0]) > half * internal)))
      return 0;
    c->depth = ((-uvsign * d) - (internal * half));
    for (int i = 0; i < 3; ++i) {
      c->pos[i] = ray.pos[i] + (c->depth * RR[i * 4 + 2]);
      c->normal[i] = uvsign * (CR[i * 4 + 2]);
    }
    return 1;
  }
  if (k > 0.f) {
    k = sqrtf(k);
    A = 1.0f / (2.f * A);
    float alpha = (-B - k) * A;
    if (alpha < 0.f) alpha = (-B + k) * A;
    if (alpha >= 0.f && alpha <= ray.p[0]) {
      for (int i = 0; i < 3; ++i) c->pos[i] = ray.pos[i] + (alpha * RR[i * 4 + 2]);
      for (int i = 0; i < 3; ++i) q[i] = c->pos[i] - cy.pos[i];
      d = q[0] * CR[2] + q[1] * CR[6] + q[2] * CR[10];
      if (d >= -half && d <= +half) {
        const float nsign = (C < 0.f) ? -1.0f : 1.0f;
        for (int i = 0; i < 3; ++i) c->normal[i] = nsign * (c->pos[i] - (cy.pos[i] + d * CR[i * 4 + 2]));
        safe_normalize3(c->normal);
        c->depth = alpha;
        return 1;
      }
    }
  }
  return 0;
}

// dCollideCylinderBox (ode/src/collision_cylinder_box.cpp:44-1036): separating
// axes over the box faces, the cylinder axis, their cross products, the box
// vertices and the box edges against both rims; then the cylinder's side edge
// clipped by the box, or the box face clipped by the rim's octagon. Out of line
// (its scratch stays out of the callers' registers).
struct CylBox {
  float cpos[3], caxis[3], crad, clen;
  float bhalf[3], bv[8][3];
  float diff[3], normal[3], best_depth, best_rb, best_rc;
  int best_axis;
};

// dMatrix3Inv (ode/src/collision_util.h:192-212), its operator precedence kept
OG_HD void cb_mat3_inv(const float* ma, float* dst) {
  const float det = ma[0] * (ma[5] * ma[10] - ma[9] * ma[6]) - ma[1] * (ma[4] * ma[10] - ma[8] * ma[6]) +
                    ma[2] * (ma[4] * ma[9] - ma[8] * ma[5]);
  if (fabsf(det) < 0.0005f) {
    for (int k = 0; k < 12; ++k) dst[k] = 0.f;
    dst[0] = dst[5] = dst[10] = 1.f;
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
  dst[3] = dst[7] = dst[11] = 0.f;
}

// _cldTestAxis (collision_cylinder_box.cpp:206-285)
OG_HD int cb_test_axis(CylBox& D, const float* bR, float* n, int iAxis) {
  const float fL = sqrtf(dot3(n, n));
  if (fL < 1e-5f) return 1;
  safe_normalize3(n);
  const float fdot1 = dot3(D.caxis, n);
  float frc;
  if (fdot1 > 1.0f || fdot1 < -1.0f) frc = D.clen * 0.5f;
  else frc = fabsf(fdot1 * (D.clen * 0.5f)) + D.crad * sqrtf(1.0f - (fdot1 * fdot1));
  float frb = 0.f;
  for (int j = 0; j < 3; ++j) {
    const float col[3] = {bR[j], bR[4 + j], bR[8 + j]};
    frb += fabsf(dot3(col, n)) * D.bhalf[j];
  }
  const float fd = dot3(D.diff, n);
  float fDepth = frc + frb;
  if (fabsf(fd) > fDepth) return 0;
  fDepth -= fabsf(fd);
  if (fDepth < D.best_depth) {
    D.best_depth = fDepth;
    D.normal[0] = n[0]; D.normal[1] = n[1]; D.normal[2] = n[2];
    D.best_axis = iAxis;
    D.best_rb = frb;
    D.best_rc = frc;
    if (fd > 0.f) { D.normal[0] = -D.normal[0]; D.normal[1] = -D.normal[1]; D.normal[2] = -D.normal[2]; }
  }
  return 1;
}

// _cldTestEdgeCircleAxis (collision_cylinder_box.cpp:289-333)
OG_HD int cb_test_edge_circle(CylBox& D, const float* bR, const float* cc, const float* v0, const float* v1,
                              int iAxis) {
  float e[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
  safe_normalize3(e);
  const float fdot2 = dot3(e, D.caxis);
  if (fabsf(fdot2) < 1e-5f) return 1;
  float t1[3] = {cc[0] - v0[0], cc[1] - v0[1], cc[2] - v0[2]};
  const float fdot1 = dot3(t1, D.caxis);
  float p[3];
  for (int i = 0; i < 3; ++i) p[i] = v0[i] + e[i] * (fdot1 / fdot2);
  float tn[3], ax[3];
  for (int i = 0; i < 3; ++i) t1[i] = cc[i] - p[i];
  cross3(tn, t1, D.caxis);
  cross3(ax, tn, e);
  return cb_test_axis(D, bR, ax, iAxis);
}

// dClipEdgeToPlane (ode/src/collision_util.cpp:471-510)
OG_HD int cb_clip_edge(float* e0, float* e1, const float* pl) {
  const float d0 = pl[0] * e0[0] + pl[1] * e0[1] + pl[2] * e0[2] + pl[3];
  const float d1 = pl[0] * e1[0] + pl[1] * e1[1] + pl[2] * e1[2] + pl[3];
  if (d0 < 0.f && d1 < 0.f) return 0;
  if (d0 > 0.f && d1 > 0.f) return 1;
  if ((d0 > 0.f && d1 < 0.f) || (d0 < 0.f && d1 > 0.f)) {
    float ip[3];
    for (int i = 0; i < 3; ++i) ip[i] = e0[i] - (e0[i] - e1[i]) * d0 / (d0 - d1);
    float* dst = (d0 < 0.f) ? e0 : e1;
    dst[0] = ip[0]; dst[1] = ip[1]; dst[2] = ip[2];
  }
  return 1;
}

// dClipPolyToPlane (ode/src/collision_util.cpp:512-553); points beyond the
// reference's 16-entry buffers (MAX_CYLBOX_CLIP_POINTS) are dropped.
constexpr int kCylBoxClip = 16;
OG_HD int cb_clip_poly(const float (*in)[3], int nin, float (*out)[3], const float* pl) {
  int n = 0;
  for (int i1 = 0, i0 = nin - 1; i1 < nin; i0 = i1, i1++) {
    const float d0 = pl[0] * in[i0][0] + pl[1] * in[i0][1] + pl[2] * in[i0][2] + pl[3];
    const float d1 = pl[0] * in[i1][0] + pl[1] * in[i1][1] + pl[2] * in[i1][2] + pl[3];
    if (d0 >= 0.f && n < kCylBoxClip) { out[n][0] = in[i0][0]; out[n][1] = in[i0][1]; out[n][2] = in[i0][2]; n++; }
    if (((d0 > 0.f && d1 < 0.f) || (d0 < 0.f && d1 > 0.f)) && n < kCylBoxClip) {
      for (int i = 0; i < 3; ++i) out[n][i] = in[i0][i] - (in[i0][i] - in[i1][i]) * d0 / (d0 - d1);
      n++;
    }
  }
  return n;
}

#if defined(__CUDACC__)
#define OG_HD_OUTLINE static __host__ __device__ __noinline__
#else
#define OG_HD_OUTLINE static
#endif
OG_HD_OUTLINE int collide_cylinder_box(const GeomView& cy, const GeomView& bx, unsigned flags, Contact* c) {
  const int maxc = (int)(flags & 0xffff);
  const float* cR = cy.R;
  const float* bR = bx.R;
  CylBox D;
  // _cldInitCylinderBox (:100-203)
  for (int i = 0; i < 3; ++i) { D.cpos[i] = cy.pos[i]; D.caxis[i] = cR[i * 4 + 2]; D.bhalf[i] = bx.p[i] * 0.5f; }
  D.crad = cy.p[0];
  D.clen = cy.p[1];
  for (int k = 0; k < 8; ++k) {
    // vertex signs: (-,+,-) (+,+,-) (-,-,-) (+,-,-) (+,+,+) (+,-,+) (-,-,+) (-,+,+)
    const float sx = (0x3Au >> k) & 1u ? 1.f : -1.f;
    const float sy = (0x93u >> k) & 1u ? 1.f : -1.f;
    const float sz = (k >= 4) ? 1.f : -1.f;
    const float v[3] = {sx * D.bhalf[0], sy * D.bhalf[1], sz * D.bhalf[2]};
    float w[3];
    mul0_331(w, bR, v);
    for (int i = 0; i < 3; ++i) D.bv[k][i] = w[i] + bx.pos[i];
  }
  for (int i = 0; i < 3; ++i) D.diff[i] = D.cpos[i] - bx.pos[i];
  // _cldTestSeparatingAxes (:336-574)
  D.best_depth = INFINITY;
  D.best_axis = 0;
  D.best_rb = D.best_rc = 0.f;
  D.normal[0] = D.normal[1] = D.normal[2] = 0.f;
  float ax[3];
  for (int j = 0; j < 3; ++j) {
    ax[0] = bR[j]; ax[1] = bR[4 + j]; ax[2] = bR[8 + j];
    if (!cb_test_axis(D, bR, ax, 1 + j)) return 0;
  }
  ax[0] = D.caxis[0]; ax[1] = D.caxis[1]; ax[2] = D.caxis[2];
  if (!cb_test_axis(D, bR, ax, 4)) return 0;
  for (int j = 0; j < 3; ++j) {
    const float col[3] = {bR[j], bR[4 + j], bR[8 + j]};
    cross3(ax, D.caxis, col);
    if (dot3(ax, ax) > 1e-6f && !cb_test_axis(D, bR, ax, 5 + j)) return 0;
  }
  for (int k = 0; k < 8; ++k) {
    float t1[3] = {D.bv[k][0] - D.cpos[0], D.bv[k][1] - D.cpos[1], D.bv[k][2] - D.cpos[2]}, t2[3];
    cross3(t2, D.caxis, t1);
    cross3(ax, D.caxis, t2);
    if (dot3(ax, ax) > 1e-6f && !cb_test_axis(D, bR, ax, 8 + k)) return 0;
  }
  // box edges (vertex pairs) against the top rim, then the bottom rim
  const unsigned char edges[12][2] = {{1, 0}, {1, 3}, {2, 3}, {2, 0}, {4, 1}, {4, 7},
                                      {0, 7}, {5, 3}, {5, 6}, {2, 6}, {4, 5}, {6, 7}};
  for (int side = 0; side < 2; ++side) {
    float cc[3];
    for (int i = 0; i < 3; ++i)
      cc[i] = (side == 0) ? D.cpos[i] + D.caxis[i] * (D.clen * 0.5f) : D.cpos[i] - D.caxis[i] * (D.clen * 0.5f);
    for (int e = 0; e < 12; ++e)
      if (!cb_test_edge_circle(D, bR, cc, D.bv[edges[e][0]], D.bv[edges[e][1]], 16 + 12 * side + e)) return 0;
  }
  if (D.best_axis == 0) return 0;
  int n = 0;
  if (fabsf(dot3(D.normal, D.caxis)) < 0.9f) {
    // _cldClipCylinderToBox (:576-717)
    const float t = dot3(D.caxis, D.normal);
    float vN[3];
    for (int i = 0; i < 3; ++i) vN[i] = D.normal[i] - D.caxis[i] * t;
    safe_normalize3(vN);
    float e0[3], e1[3];
    for (int i = 0; i < 3; ++i) {
      const float ct = D.cpos[i] + vN[i] * D.crad;
      e0[i] = ct + D.caxis[i] * (D.clen * 0.5f);
      e1[i] = ct - D.caxis[i] * (D.clen * 0.5f);
    }
    for (int i = 0; i < 3; ++i) { e0[i] -= bx.pos[i]; e1[i] -= bx.pos[i]; }
    for (int neg = 0; neg < 2; ++neg)
      for (int j = 0; j < 3; ++j) {
        float pl[4] = {bR[j], bR[4 + j], bR[8 + j], D.bhalf[j]};
        if (neg) { pl[0] = -pl[0]; pl[1] = -pl[1]; pl[2] = -pl[2]; }
        if (!cb_clip_edge(e0, e1, pl)) return 0;
      }
    float d0 = D.best_rb + dot3(e0, D.normal);
    float d1 = D.best_rb + dot3(e1, D.normal);
    if (d0 < 0.f) d0 = 0.f;
    if (d1 < 0.f) d1 = 0.f;
    for (int i = 0; i < 3; ++i) { e0[i] += bx.pos[i]; e1[i] += bx.pos[i]; }
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
  // _cldClipBoxToCylinder (:720-983)
  float ccp[3], cn_z;
  if (dot3(D.caxis, D.normal) > 0.f) {
    for (int i = 0; i < 3; ++i) ccp[i] = D.cpos[i] + D.caxis[i] * (D.clen * 0.5f);
    cn_z = -1.0f;
  } else {
    for (int i = 0; i < 3; ++i) ccp[i] = D.cpos[i] - D.caxis[i] * (D.clen * 0.5f);
    cn_z = 1.0f;
  }
  float inv[12], vNr[3];
  cb_mat3_inv(bR, inv);
  mul0_331(vNr, inv, D.normal);
  const float an[3] = {fabsf(vNr[0]), fabsf(vNr[1]), fabsf(vNr[2])};
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
  float ctr[3];
  for (int i = 0; i < 3; ++i) {
    const float col = bR[i * 4 + iB0];
    ctr[i] = (vNr[iB0] > 0.f) ? bx.pos[i] - D.bhalf[iB0] * col : bx.pos[i] + D.bhalf[iB0] * col;
  }
  float A1[kCylBoxClip][3], A2[kCylBoxClip][3], pts[4][3];
  const float h1 = D.bhalf[iB1], h2 = D.bhalf[iB2];
  for (int i = 0; i < 3; ++i) {
    const float a1 = bR[i * 4 + iB1], a2 = bR[i * 4 + iB2];
    pts[0][i] = ctr[i] + h1 * a1 - h2 * a2;
    pts[1][i] = ctr[i] - h1 * a1 - h2 * a2;
    pts[2][i] = ctr[i] - h1 * a1 + h2 * a2;
    pts[3][i] = ctr[i] + h1 * a1 + h2 * a2;
  }
  cb_mat3_inv(cR, inv);
  for (int k = 0; k < 4; ++k) {
    const float t[3] = {pts[k][0] - ccp[0], pts[k][1] - ccp[1], pts[k][2] - ccp[2]};
    mul0_331(pts[k], inv, t);
  }
  float pl[4] = {0.f, 0.f, cn_z, 0.f};
  int n1 = cb_clip_poly(pts, 4, A1, pl), n2 = 0;
  // the rim as an octagon: plane normals -(cos, sin) of pi/8 + k pi/4
  float ang = (float)(3.14159265358979323846 / 8);
  const float inc = ang * 2.0f;
  for (int seg = 0; seg < 8; ++seg) {
    pl[0] = -cosf(ang); pl[1] = -sinf(ang); pl[2] = 0.f; pl[3] = D.crad;
    ang += inc;
    if (seg % 2 == 0) n2 = cb_clip_poly(A1, n1, A2, pl);
    else n1 = cb_clip_poly(A2, n2, A1, pl);
  }
  for (int k = 0; k < n1; ++k) {   // after 8 segments the result is in A1
    float p[3];
    mul0_331(p, cR, A1[k]);
    for (int i = 0; i < 3; ++i) p[i] += ccp[i];
    const float t[3] = {p[0] - D.cpos[0], p[1] - D.cpos[1], p[2] - D.cpos[2]};
    const float dep = D.best_rc - dot3(t, D.normal);
    if (dep > 0.f) {
      c[n].depth = dep;
      for (int i = 0; i < 3; ++i) { c[n].normal[i] = -D.normal[i]; c[n].pos[i] = p[i]; }
      if (++n == maxc) break;
    }
  }
  return n;
}

// Collider table for this path (ode/src/collision_kernel.cpp:167-268): returns
// a collider id and whether the call runs with the geoms swapped (in which case
// dCollide negates the normals, :319-335).
enum { CL_NONE = 0, CL_SS, CL_SB, CL_SP, CL_BB, CL_BP, CL_CP, CL_HF, CL_CS, CL_CB, CL_CC,
       CL_RS, CL_RB, CL_RC, CL_RP, CL_YS, CL_YB, CL_YP, CL_RY };
OG_HD int collider_of(int t1, int t2, int* reverse) {
  *reverse = 0;
  auto is = [&](int a, int b) { return t1 == a && t2 == b; };
  if (is(G_SPHERE, G_SPHERE)) return CL_SS;
  if (is(G_SPHERE, G_BOX)) return CL_SB;
  if (is(G_BOX, G_SPHERE)) { *reverse = 1; return CL_SB; }
  if (is(G_SPHERE, G_PLANE)) return CL_SP;
  if (is(G_PLANE, G_SPHERE)) { *reverse = 1; return CL_SP; }
  if (is(G_BOX, G_BOX)) return CL_BB;
  if (is(G_BOX, G_PLANE)) return CL_BP;
  if (is(G_PLANE, G_BOX)) { *reverse = 1; return CL_BP; }
  if (is(G_CAPSULE, G_SPHERE)) return CL_CS;
  if (is(G_SPHERE, G_CAPSULE)) { *reverse = 1; return CL_CS; }
  if (is(G_CAPSULE, G_BOX)) return CL_CB;
  if (is(G_BOX, G_CAPSULE)) { *reverse = 1; return CL_CB; }
  if (is(G_CAPSULE, G_CAPSULE)) return CL_CC;
  if (is(G_CAPSULE, G_PLANE)) return CL_CP;
  if (is(G_PLANE, G_CAPSULE)) { *reverse = 1; return CL_CP; }
  if (is(G_RAY, G_SPHERE)) return CL_RS;
  if (is(G_SPHERE, G_RAY)) { *reverse = 1; return CL_RS; }
  if (is(G_RAY, G_BOX)) return CL_RB;
  if (is(G_BOX, G_RAY)) { *reverse = 1; return CL_RB; }
  if (is(G_RAY, G_CAPSULE)) return CL_RC;
  if (is(G_CAPSULE, G_RAY)) { *reverse = 1; return CL_RC; }
  if (is(G_RAY, G_PLANE)) return CL_RP;
  if (is(G_PLANE, G_RAY)) { *reverse = 1; return CL_RP; }
  // cylinder-cylinder and capsule-cylinder need libccd (collision_kernel.cpp:215-220): no collider
  if (is(G_CYLINDER, G_SPHERE)) return CL_YS;
  if (is(G_SPHERE, G_CYLINDER)) { *reverse = 1; return CL_YS; }
  if (is(G_CYLINDER, G_BOX)) return CL_YB;
  if (is(G_BOX, G_CYLINDER)) { *reverse = 1; return CL_YB; }
  if (is(G_CYLINDER, G_PLANE)) return CL_YP;
  if (is(G_PLANE, G_CYLINDER)) { *reverse = 1; return CL_YP; }
  if (is(G_RAY, G_CYLINDER)) return CL_RY;
  if (is(G_CYLINDER, G_RAY)) { *reverse = 1; return CL_RY; }
  auto hf_other = [](int t) {
    return t == G_SPHERE || t == G_BOX || t == G_CAPSULE || t == G_CYLINDER || t == G_RAY;
  };
  if (t1 == G_HEIGHTFIELD && hf_other(t2)) return CL_HF;
  if (t2 == G_HEIGHTFIELD && hf_other(t1)) { *reverse = 1; return CL_HF; }
  return CL_NONE;
}

// dCollide for the classes above without a heightfield (the heightfield has
// its own entry in heightfield.cuh). `c` must hold 4 (or flags & 0xffff, at
// most 8) contacts.
OG_HD int collide_primitive(const GeomView& g1, const GeomView& g2, unsigned flags, Contact* c) {
  if ((flags & 0xffff) == 0) return 0;
  int rev;
  const int id = collider_of(g1.type, g2.type, &rev);
  const GeomView& a = rev ? g2 : g1;
  const GeomView& b = rev ? g1 : g2;
  int n = 0;
  switch (id) {
    case CL_SS: n = collide_spheres(a.pos, a.p[0], b.pos, b.p[0], c); break;
    case CL_SB: n = collide_sphere_box(a, b, c); break;
    case CL_SP: n = collide_sphere_plane(a, b, c); break;
    case CL_BB: n = collide_box_box(a, b, flags, c); break;
    case CL_BP: n = collide_box_plane(a, b, flags, c); break;
    case CL_CP: n = collide_capsule_plane(a, b, flags, c); break;
    case CL_CS: n = collide_capsule_sphere(a, b, c); break;
    case CL_CB: n = collide_capsule_box(a, b, c); break;
    case CL_CC: n = collide_capsule_capsule(a, b, flags, c); break;
    case CL_RS: n = ray_sphere_helper(a, b.pos, b.p[0], c, 0); break;
    case CL_RB: n = collide_ray_box(a, b, c); break;
    case CL_RC: n = collide_ray_capsule(a, b, c); break;
    case CL_RP: n = collide_ray_plane(a, b, c); break;
    case CL_YS: n = collide_cylinder_sphere(a, b, c); break;
    case CL_YB: n = collide_cylinder_box(a, b, flags, c); break;
    case CL_YP: n = collide_cylinder_plane(a, b, flags, c); break;
    case CL_RY: n = collide_ray_cylinder(a, b, c); break;
    default: n = 0;
  }
  if (rev)
    for (int i = 0; i < n; ++i) {
      c[i].normal[0] = -c[i].normal[0]; c[i].normal[1] = -c[i].normal[1]; c[i].normal[2] = -c[i].normal[2];
    }
  return n;
}

}  // namespace og
