// host_setup.hpp -- FP64 host-side object setup done once at upload time:
// what ODE's setter calls compute when a scene is built (dBodySetQuaternion,
// dBodySetMass, dCreatePlane, dJointAttach + dJointSet*Anchor/Axis/Param).
// None of this runs per step.
#pragma once
#include <cmath>
#include <cstring>

namespace og_host {

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline void cross3(double* r, const double* a, const double* b) {
  double r0 = a[1] * b[2] - a[2] * b[1], r1 = a[2] * b[0] - a[0] * b[2], r2 = a[0] * b[1] - a[1] * b[0];
  r[0] = r0; r[1] = r1; r[2] = r2;
}
// R is 3x4 row-major as in ODE
inline void mul0_331(double* res, const double* A, const double* b) {
  double r0 = dot3(A, b), r1 = dot3(A + 4, b), r2 = dot3(A + 8, b);
  res[0] = r0; res[1] = r1; res[2] = r2;
}
inline void mul1_331(double* res, const double* A, const double* b) {
  double r0 = A[0] * b[0] + A[4] * b[1] + A[8] * b[2];
  double r1 = A[1] * b[0] + A[5] * b[1] + A[9] * b[2];
  double r2 = A[2] * b[0] + A[6] * b[1] + A[10] * b[2];
  res[0] = r0; res[1] = r1; res[2] = r2;
}
inline void normalize4(double* a) {
  double l = dot3(a, a) + a[3] * a[3];
  if (l > 0) { l = 1.0 / std::sqrt(l); for (int i = 0; i < 4; ++i) a[i] *= l; }
  else { a[0] = 1; a[1] = a[2] = a[3] = 0; }
}
// _dSafeNormalize3 (ode/src/odemath.cpp:42-83)
inline void safe_normalize3(double* a) {
  double aa[3] = {std::fabs(a[0]), std::fabs(a[1]), std::fabs(a[2])};
  int idx;
  if (aa[1] > aa[0]) idx = (aa[2] > aa[1]) ? 2 : 1;
  else if (aa[2] > aa[0]) idx = 2;
  else {
    if (aa[0] <= 0) { a[0] = 1; a[1] = 0; a[2] = 0; return; }
    idx = 0;
  }
  a[0] /= aa[idx]; a[1] /= aa[idx]; a[2] /= aa[idx];
  double l = 1.0 / std::sqrt(dot3(a, a));
  a[0] *= l; a[1] *= l; a[2] *= l;
}
// dRfromQ (ode/src/rotation.cpp:236-255)
inline void r_from_q(double* R, const double* q) {
  double qq1 = 2 * q[1] * q[1], qq2 = 2 * q[2] * q[2], qq3 = 2 * q[3] * q[3];
  R[0] = 1 - qq2 - qq3; R[1] = 2 * (q[1] * q[2] - q[0] * q[3]); R[2] = 2 * (q[1] * q[3] + q[0] * q[2]); R[3] = 0;
  R[4] = 2 * (q[1] * q[2] + q[0] * q[3]); R[5] = 1 - qq1 - qq3; R[6] = 2 * (q[2] * q[3] - q[0] * q[1]); R[7] = 0;
  R[8] = 2 * (q[1] * q[3] - q[0] * q[2]); R[9] = 2 * (q[2] * q[3] + q[0] * q[1]); R[10] = 1 - qq1 - qq2; R[11] = 0;
}
// dQMultiply0 / dQMultiply1 (ode/src/rotation.cpp:191-208)
inline void qmul0(double* qa, const double* qb, const double* qc) {
  qa[0] = qb[0] * qc[0] - qb[1] * qc[1] - qb[2] * qc[2] - qb[3] * qc[3];
  qa[1] = qb[0] * qc[1] + qb[1] * qc[0] + qb[2] * qc[3] - qb[3] * qc[2];
  qa[2] = qb[0] * qc[2] + qb[2] * qc[0] + qb[3] * qc[1] - qb[1] * qc[3];
  qa[3] = qb[0] * qc[3] + qb[3] * qc[0] + qb[1] * qc[2] - qb[2] * qc[1];
}
inline void qmul1(double* qa, const double* qb, const double* qc) {
  qa[0] = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
  qa[1] = qb[0] * qc[1] - qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
  qa[2] = qb[0] * qc[2] - qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
  qa[3] = qb[0] * qc[3] - qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
}

// dQMultiply2 / dQMultiply3 (ode/src/rotation.cpp:211-226)
inline void qmul2(double* qa, const double* qb, const double* qc) {
  qa[0] = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
  qa[1] = -qb[0] * qc[1] + qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
  qa[2] = -qb[0] * qc[2] + qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
  qa[3] = -qb[0] * qc[3] + qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
}
inline void qmul3(double* qa, const double* qb, const double* qc) {
  qa[0] = qb[0] * qc[0] - qb[1] * qc[1] - qb[2] * qc[2] - qb[3] * qc[3];
  qa[1] = -qb[0] * qc[1] - qb[1] * qc[0] + qb[2] * qc[3] - qb[3] * qc[2];
  qa[2] = -qb[0] * qc[2] - qb[2] * qc[0] + qb[3] * qc[1] - qb[1] * qc[3];
  qa[3] = -qb[0] * qc[3] - qb[3] * qc[0] + qb[1] * qc[2] - qb[2] * qc[1];
}
// getHingeAngleFromRelativeQuat (ode/src/joints/joint.cpp:381-420)
inline double hinge_angle_from_qrel(const double* qrel, const double* axis) {
  const double cost2 = qrel[0];
  const double sint2 = std::sqrt(qrel[1] * qrel[1] + qrel[2] * qrel[2] + qrel[3] * qrel[3]);
  double theta = (dot3(qrel + 1, axis) >= 0) ? 2 * std::atan2(sint2, cost2) : 2 * std::atan2(sint2, -cost2);
  if (theta > M_PI) theta -= 2 * M_PI;
  return -theta;
}

// 3x3 SPD inverse through a Cholesky factorisation, the method dBodySetMass
// uses (dInvertPDMatrix, ode/src/matrix.cpp:121-230). A, out: 3x3 row-major.
inline bool invert_pd3(const double* A, double* out) {
  double L[9], rec[3];
  std::memcpy(L, A, sizeof(L));
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < i; ++j) {
      double s = L[i * 3 + j];
      for (int k = 0; k < j; ++k) s -= L[i * 3 + k] * L[j * 3 + k];
      L[i * 3 + j] = s * rec[j];
    }
    double s = L[i * 3 + i];
    for (int k = 0; k < i; ++k) s -= L[i * 3 + k] * L[i * 3 + k];
    if (s <= 0) return false;
    L[i * 3 + i] = std::sqrt(s);
    rec[i] = 1.0 / L[i * 3 + i];
  }
  for (int c = 0; c < 3; ++c) {
    double x[3] = {0, 0, 0}, y[3];
    x[c] = 1;
    for (int r = 0; r < 3; ++r) {
      double s = 0;
      for (int k = 0; k < r; ++k) s += L[r * 3 + k] * y[k];
      y[r] = (x[r] - s) / L[r * 3 + r];
    }
    for (int r = 2; r >= 0; --r) {
      double s = 0;
      for (int k = r + 1; k < 3; ++k) s += L[k * 3 + r] * x[k];
      x[r] = (y[r] - s) / L[r * 3 + r];
    }
    for (int r = 0; r < 3; ++r) out[r * 3 + c] = x[r];
  }
  return true;
}

// dRFrom2Axes (ode/src/rotation.cpp:94-133); a zero-length input leaves R as given
inline void r_from_2axes(double* R, double ax, double ay, double az, double bx, double by, double bz) {
  double l = std::sqrt(ax * ax + ay * ay + az * az);
  if (l <= 0) return;
  l = 1.0 / l;
  ax *= l; ay *= l; az *= l;
  const double k = ax * bx + ay * by + az * bz;
  bx -= k * ax; by -= k * ay; bz -= k * az;
  l = std::sqrt(bx * bx + by * by + bz * bz);
  if (l <= 0) return;
  l = 1.0 / l;
  bx *= l; by *= l; bz *= l;
  R[0] = ax; R[4] = ay; R[8] = az;
  R[1] = bx; R[5] = by; R[9] = bz;
  R[2] = -by * az + ay * bz; R[6] = -bz * ax + az * bx; R[10] = -bx * ay + ax * by;
  R[3] = 0; R[7] = 0; R[11] = 0;
}
// dQfromR (ode/src/rotation.cpp:258-306)
inline void q_from_r(double* q, const double* R) {
  const double tr = R[0] + R[5] + R[10];
  double s;
  if (tr >= 0) {
    s = std::sqrt(tr + 1);
    q[0] = 0.5 * s;
    s = 0.5 * (1.0 / s);
    q[1] = (R[9] - R[6]) * s; q[2] = (R[2] - R[8]) * s; q[3] = (R[4] - R[1]) * s;
    return;
  }
  int c;
  if (R[5] > R[0]) c = (R[10] > R[5]) ? 2 : 1;
  else c = (R[10] > R[0]) ? 2 : 0;
  if (c == 0) {
    s = std::sqrt((R[0] - (R[5] + R[10])) + 1);
    q[1] = 0.5 * s;
    s = 0.5 * (1.0 / s);
    q[2] = (R[1] + R[4]) * s; q[3] = (R[8] + R[2]) * s; q[0] = (R[9] - R[6]) * s;
  } else if (c == 1) {
    s = std::sqrt((R[5] - (R[10] + R[0])) + 1);
    q[2] = 0.5 * s;
    s = 0.5 * (1.0 / s);
    q[3] = (R[6] + R[9]) * s; q[1] = (R[1] + R[4]) * s; q[0] = (R[2] - R[8]) * s;
  } else {
    s = std::sqrt((R[10] - (R[0] + R[5])) + 1);
    q[3] = 0.5 * s;
    s = 0.5 * (1.0 / s);
    q[1] = (R[8] + R[2]) * s; q[2] = (R[6] + R[9]) * s; q[0] = (R[4] - R[1]) * s;
  }
}

struct HBody { double pos[3], q[4], R[12]; };

// Joint geometry computed by the setters (ode/src/joints/joint.cpp:260-322,
// hinge.cpp:378-396, hinge2.cpp:97-106 and :184-210, slider.cpp:355-398,
// universal.cpp:365-393, fixed.cpp:110-132).
struct HJoint {
  int b1, b2, reverse;
  double anchor1[4], anchor2[4], axis1[4], axis2[4], qrel[4], v1[4], v2[4];
  double offset[4];   // slider, fixed
  double qrel2[4];    // universal (qrel holds qrel1)
  double c0, s0;
  // angular motor (ode/src/joints/amotor.h)
  int am_num, am_mode, am_rel[3];
  double am_axis[3][4], am_ref1[4], am_ref2[4], am_angle[3];
};

inline void attach(HJoint& J, int b1, int b2) {
  if (b1 < 0) { b1 = b2; b2 = -1; J.reverse = 1; } else J.reverse = 0;
  J.b1 = b1; J.b2 = b2;
}
inline void set_anchors(HJoint& J, const HBody* B, double x, double y, double z, double* a1, double* a2) {
  if (J.b1 >= 0) {
    const HBody& B1 = B[J.b1];
    double q[3] = {x - B1.pos[0], y - B1.pos[1], z - B1.pos[2]};
    mul1_331(a1, B1.R, q);
    if (J.b2 >= 0) {
      const HBody& B2 = B[J.b2];
      double q2[3] = {x - B2.pos[0], y - B2.pos[1], z - B2.pos[2]};
      mul1_331(a2, B2.R, q2);
    } else { a2[0] = x; a2[1] = y; a2[2] = z; }
  }
  a1[3] = 0; a2[3] = 0;
}
inline void set_axes(HJoint& J, const HBody* B, double x, double y, double z, double* ax1, double* ax2) {
  if (J.b1 < 0) return;
  double q[3] = {x, y, z};
  safe_normalize3(q);
  if (ax1) { mul1_331(ax1, B[J.b1].R, q); ax1[3] = 0; }
  if (ax2) {
    if (J.b2 >= 0) mul1_331(ax2, B[J.b2].R, q);
    else { ax2[0] = x; ax2[1] = y; ax2[2] = z; }
    ax2[3] = 0;
  }
}
inline void hinge_qrel(HJoint& J, const HBody* B) {
  if (J.b1 < 0) return;
  const double* q1 = B[J.b1].q;
  if (J.b2 >= 0) qmul1(J.qrel, q1, B[J.b2].q);
  else { J.qrel[0] = q1[0]; J.qrel[1] = -q1[1]; J.qrel[2] = -q1[2]; J.qrel[3] = -q1[3]; }
}
inline void hinge2_axis_info(HJoint& J, const HBody* B) {
  double ax1[3], ax2[3], axc[3];
  mul0_331(ax1, B[J.b1].R, J.axis1);
  mul0_331(ax2, B[J.b2].R, J.axis2);
  cross3(axc, ax1, ax2);
  J.s0 = std::sqrt(dot3(axc, axc));
  J.c0 = dot3(ax1, ax2);
}
inline void hinge2_make_v(HJoint& J, const HBody* B) {
  if (J.b1 < 0 || J.b2 < 0) return;
  double ax1[3], ax2[3], v[3];
  mul0_331(ax1, B[J.b1].R, J.axis1);
  mul0_331(ax2, B[J.b2].R, J.axis2);
  if ((ax1[0] == 0 && ax1[1] == 0 && ax1[2] == 0) || (ax2[0] == 0 && ax2[1] == 0 && ax2[2] == 0) ||
      (ax1[0] == ax2[0] && ax1[1] == ax2[1] && ax1[2] == ax2[2]))
    return;
  double k = dot3(ax1, ax2);
  for (int i = 0; i < 3; ++i) ax2[i] -= k * ax1[i];
  safe_normalize3(ax2);
  cross3(v, ax1, ax2);
  mul1_331(J.v1, B[J.b1].R, ax2);
  mul1_331(J.v2, B[J.b1].R, v);
}

// Initial relative rotation body1 -> body2, or env -> body1, of the hinge,
// slider and fixed joints (hinge.cpp:378-396, slider.cpp:355-376, fixed.cpp:193-210)
inline void initial_qrel(HJoint& J, const HBody* B) { hinge_qrel(J, B); }

// dxJointSlider::computeOffset (ode/src/joints/slider.cpp:380-398)
inline void slider_offset(HJoint& J, const HBody* B) {
  if (J.b2 >= 0) {
    double c[3];
    for (int i = 0; i < 3; ++i) c[i] = B[J.b1].pos[i] - B[J.b2].pos[i];
    mul1_331(J.offset, B[J.b2].R, c);
  } else if (J.b1 >= 0) {
    for (int i = 0; i < 3; ++i) J.offset[i] = B[J.b1].pos[i];
  }
}

// dJointSetFixed's offset (ode/src/joints/fixed.cpp:110-132): body 2 -> body 1
// in body 1's frame, unlike the slider's.
inline void fixed_offset(HJoint& J, const HBody* B) {
  if (J.b1 < 0) return;
  if (J.b2 >= 0) {
    double ofs[3];
    for (int i = 0; i < 3; ++i) ofs[i] = B[J.b1].pos[i] - B[J.b2].pos[i];
    mul1_331(J.offset, B[J.b1].R, ofs);
  } else {
    for (int i = 0; i < 3; ++i) J.offset[i] = B[J.b1].pos[i];
  }
}

// dxJointUniversal::computeInitialRelativeRotations (ode/src/joints/universal.cpp:365-393)
inline void universal_qrels(HJoint& J, const HBody* B) {
  if (J.b1 < 0) return;
  double ax1[3], ax2[3], R[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, qcross[4];
  mul0_331(ax1, B[J.b1].R, J.axis1);
  if (J.b2 >= 0) mul0_331(ax2, B[J.b2].R, J.axis2);
  else { ax2[0] = J.axis2[0]; ax2[1] = J.axis2[1]; ax2[2] = J.axis2[2]; }
  r_from_2axes(R, ax1[0], ax1[1], ax1[2], ax2[0], ax2[1], ax2[2]);
  q_from_r(qcross, R);
  qmul1(J.qrel, B[J.b1].q, qcross);
  r_from_2axes(R, ax2[0], ax2[1], ax2[2], ax1[0], ax1[1], ax1[2]);
  q_from_r(qcross, R);
  if (J.b2 >= 0) qmul1(J.qrel2, B[J.b2].q, qcross);
  else for (int i = 0; i < 4; ++i) J.qrel2[i] = qcross[i];
}

// dxJointUniversal::getAxes (ode/src/joints/universal.cpp:55-70)
inline void universal_axes(const HJoint& J, const HBody* B, double* ax1, double* ax2) {
  mul0_331(ax1, B[J.b1].R, J.axis1);
  if (J.b2 >= 0) mul0_331(ax2, B[J.b2].R, J.axis2);
  else { ax2[0] = J.axis2[0]; ax2[1] = J.axis2[1]; ax2[2] = J.axis2[2]; }
}
// dxJointUniversal::getAngles (ode/src/joints/universal.cpp:73-167)
inline void universal_angles(const HJoint& J, const HBody* B, double* angle1, double* angle2) {
  if (J.b1 < 0) { *angle1 = 0; *angle2 = 0; return; }
  double ax1[3], ax2[3], R[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, qcross[4], qq[4], qrel[4], qcross2[4];
  universal_axes(J, B, ax1, ax2);
  r_from_2axes(R, ax1[0], ax1[1], ax1[2], ax2[0], ax2[1], ax2[2]);
  q_from_r(qcross, R);
  qmul1(qq, B[J.b1].q, qcross);
  qmul2(qrel, qq, J.qrel);
  *angle1 = hinge_angle_from_qrel(qrel, J.axis1);
  qrel[0] = 0;
  qrel[1] = ax1[0] + ax2[0];
  qrel[2] = ax1[1] + ax2[1];
  qrel[3] = ax1[2] + ax2[2];
  const double l = 1.0 / std::sqrt(qrel[1] * qrel[1] + qrel[2] * qrel[2] + qrel[3] * qrel[3]);
  qrel[1] *= l; qrel[2] *= l; qrel[3] *= l;
  qmul0(qcross2, qrel, qcross);
  if (J.b2 >= 0) {
    qmul1(qq, B[J.b2].q, qcross2);
    qmul2(qrel, qq, J.qrel2);
  } else {
    qmul2(qrel, qcross2, J.qrel2);
  }
  *angle2 = -hinge_angle_from_qrel(qrel, J.axis2);
}
// dxJointUniversal::getAngle1 / getAngle2 (ode/src/joints/universal.cpp:170-255):
// angle 2 here uses the cross frame dRFrom2Axes(ax2, ax1), unlike getAngles
inline double universal_angle1(const HJoint& J, const HBody* B) {
  double a1, a2;
  universal_angles(J, B, &a1, &a2);
  return a1;
}
inline double universal_angle2(const HJoint& J, const HBody* B) {
  if (J.b1 < 0) return 0;
  double ax1[3], ax2[3], R[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, qcross[4], qq[4], qrel[4];
  universal_axes(J, B, ax1, ax2);
  r_from_2axes(R, ax2[0], ax2[1], ax2[2], ax1[0], ax1[1], ax1[2]);
  q_from_r(qcross, R);
  if (J.b2 >= 0) {
    qmul1(qq, B[J.b2].q, qcross);
    qmul2(qrel, qq, J.qrel2);
  } else {
    qmul2(qrel, qcross, J.qrel2);
  }
  return -hinge_angle_from_qrel(qrel, J.axis2);
}
// dJointGetSliderPosition (ode/src/joints/slider.cpp:42-79)
inline double slider_position(const HJoint& J, const HBody* B) {
  double ax1[3], q[3];
  mul0_331(ax1, B[J.b1].R, J.axis1);
  if (J.b2 >= 0) {
    mul0_331(q, B[J.b2].R, J.offset);
    for (int i = 0; i < 3; ++i) q[i] = B[J.b1].pos[i] - q[i] - B[J.b2].pos[i];
  } else {
    for (int i = 0; i < 3; ++i) q[i] = B[J.b1].pos[i] - J.offset[i];
    if (J.reverse) { ax1[0] = -ax1[0]; ax1[1] = -ax1[1]; ax1[2] = -ax1[2]; }
  }
  return dot3(ax1, q);
}

// dxJointAMotor::setEulerReferenceVectors (ode/src/joints/amotor.cpp:148-181);
// without a second body the reference adds to reference2 on every call.
inline void amotor_euler_refs(HJoint& J, const HBody* B) {
  if (J.b1 < 0) return;
  if (J.b2 >= 0) {
    double r[3];
    mul0_331(r, B[J.b2].R, J.am_axis[2]);
    mul1_331(J.am_ref1, B[J.b1].R, r);
    mul0_331(r, B[J.b1].R, J.am_axis[0]);
    mul1_331(J.am_ref2, B[J.b2].R, r);
  } else {
    double r[4] = {J.am_axis[2][0], J.am_axis[2][1], J.am_axis[2][2], J.am_axis[2][3]};
    mul1_331(J.am_ref1, B[J.b1].R, r);
    mul0_331(r, B[J.b1].R, J.am_axis[0]);
    for (int k = 0; k < 4; ++k) J.am_ref2[k] += r[k];
  }
}
// dJointSetAMotorMode / NumAxes / Axis (ode/src/joints/amotor.cpp:260-323, :350-363)
inline void amotor_set_mode(HJoint& J, const HBody* B, int mode) {
  J.am_mode = mode;
  if (mode == 1) { J.am_num = 3; amotor_euler_refs(J, B); }
}
inline void amotor_set_num(HJoint& J, int num) {
  if (J.am_mode == 1) J.am_num = 3;
  else J.am_num = num < 0 ? 0 : (num > 3 ? 3 : num);
}
inline void amotor_set_axis(HJoint& J, const HBody* B, int anum, int rel, double x, double y, double z) {
  if (anum < 0) anum = 0;
  if (anum > 2) anum = 2;
  if (J.b2 < 0 && rel == 2) rel = 1;
  J.am_rel[anum] = rel;
  double r[4] = {x, y, z, 0};
  double* a = J.am_axis[anum];
  if (rel > 0) {
    if (rel == 1) mul1_331(a, B[J.b1].R, r);
    else if (J.b2 >= 0) mul1_331(a, B[J.b2].R, r);
    else for (int k = 0; k < 4; ++k) a[k] = r[k];
  } else {
    a[0] = r[0]; a[1] = r[1]; a[2] = r[2];
  }
  safe_normalize3(a);
  if (J.am_mode == 1) amotor_euler_refs(J, B);
}

// The setter sequence a scene's joint goes through: dJointAttach, then
//   ball:   dJointSetBallAnchor
//   hinge:  dJointSetHingeAnchor, dJointSetHingeAxis
//   hinge2: dJointSetHinge2Anchor, dJointSetHinge2Axis1, dJointSetHinge2Axis2
//   slider: dJointSetSliderAxis
//   universal: dJointSetUniversalAnchor, dJointSetUniversalAxis1, dJointSetUniversalAxis2
//   fixed:  dJointSetFixed
//   amotor: dJointSetAMotorMode, dJointSetAMotorNumAxes, dJointSetAMotorAxis
//           (axes 0..num-1 in user mode, 0 and 2 in Euler mode), the angles of
//           user mode (dJointSetAMotorAngle); jp is its parameter block
// (with the attach-time setRelativeValues of hinge2, hinge2.cpp:425-448; the
// slider's and universal's are overwritten in full by their setters).
inline void setup_joint(int type, HJoint& J, const HBody* B, int b1, int b2, const double* a,
                        const double* x1, const double* x2, const double* jp = nullptr) {
  std::memset(&J, 0, sizeof(J));
  J.axis1[0] = 1;
  if (type == 6) { J.axis2[1] = 1; J.v1[0] = 1; J.v2[1] = 1; }
  else if (type == 5) J.axis2[1] = 1;
  else if (type == 2) J.axis2[0] = 1;
  attach(J, b1, b2);
  if (type == 1) {
    set_anchors(J, B, a[0], a[1], a[2], J.anchor1, J.anchor2);
  } else if (type == 2) {
    set_anchors(J, B, a[0], a[1], a[2], J.anchor1, J.anchor2);
    hinge_qrel(J, B);
    set_axes(J, B, x1[0], x1[1], x1[2], J.axis1, J.axis2);
    hinge_qrel(J, B);
  } else if (type == 6) {
    if (J.b1 >= 0 && J.b2 >= 0) {
      double an[3], ax[3];
      mul0_331(an, B[J.b1].R, J.anchor1);
      for (int i = 0; i < 3; ++i) an[i] += B[J.b1].pos[i];
      set_anchors(J, B, an[0], an[1], an[2], J.anchor1, J.anchor2);
      mul0_331(ax, B[J.b1].R, J.axis1);
      set_axes(J, B, ax[0], ax[1], ax[2], J.axis1, nullptr);
      mul0_331(ax, B[J.b2].R, J.axis2);
      set_axes(J, B, ax[0], ax[1], ax[2], nullptr, J.axis2);
      hinge2_axis_info(J, B);
      hinge2_make_v(J, B);
      set_anchors(J, B, a[0], a[1], a[2], J.anchor1, J.anchor2);
      hinge2_make_v(J, B);
      set_axes(J, B, x1[0], x1[1], x1[2], J.axis1, nullptr);
      hinge2_axis_info(J, B);
      hinge2_make_v(J, B);
      set_axes(J, B, x2[0], x2[1], x2[2], nullptr, J.axis2);
      hinge2_axis_info(J, B);
      hinge2_make_v(J, B);
    }
  } else if (type == 3) {
    set_axes(J, B, x1[0], x1[1], x1[2], J.axis1, nullptr);
    slider_offset(J, B);
    initial_qrel(J, B);
  } else if (type == 5) {
    set_anchors(J, B, a[0], a[1], a[2], J.anchor1, J.anchor2);
    universal_qrels(J, B);
    // on a reversed joint axis 1 of the API is the second body axis and v.v.
    if (J.reverse) set_axes(J, B, x1[0], x1[1], x1[2], nullptr, J.axis2);
    else set_axes(J, B, x1[0], x1[1], x1[2], J.axis1, nullptr);
    universal_qrels(J, B);
    if (J.reverse) set_axes(J, B, x2[0], x2[1], x2[2], J.axis1, nullptr);
    else set_axes(J, B, x2[0], x2[1], x2[2], nullptr, J.axis2);
    universal_qrels(J, B);
  } else if (type == 7) {
    fixed_offset(J, B);
    initial_qrel(J, B);
  } else if (type == 9 && jp && J.b1 >= 0) {
    const int mode = (int)jp[1];
    amotor_set_mode(J, B, mode);
    amotor_set_num(J, (int)jp[0]);
    const double* ax[3] = {a, x1, x2};
    for (int i = 0; i < 3; ++i)
      if (mode == 1 ? i != 1 : i < J.am_num) amotor_set_axis(J, B, i, (int)jp[2 + i], ax[i][0], ax[i][1], ax[i][2]);
    if (mode == 0)
      for (int i = 0; i < J.am_num; ++i) J.am_angle[i] = jp[32 + i];
  }
}

}  // namespace og_host
