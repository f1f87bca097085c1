// joints.cuh -- FP32 joint Jacobian assembly (getInfo1 / getInfo2) on the device.
//
// Rows are written straight into the row store (see engine.cuh: 32 floats per
// row, J in words 0..11, c/cfm/lo/hi/findex in words 24..28), which plays the
// role of ODE's Info2 arrays (ode/src/joints/joint.h:86-118, rowskip = 12 in
// dxQuickStepper, ode/src/quickstep.cpp:768-771).
#pragma once
#include "dmath.cuh"
#include "engine_types.cuh"

namespace og {

struct Info2 {
  float fps, erp;
  float* rows;   // first row of this joint
  int fbase;     // its index in the world's row store: findex is stored absolute
  OG_D float& J1l(int r, int k) { return rows[r * kRowWords + k]; }
  OG_D float& J1a(int r, int k) { return rows[r * kRowWords + 3 + k]; }
  OG_D float& J2l(int r, int k) { return rows[r * kRowWords + 6 + k]; }
  OG_D float& J2a(int r, int k) { return rows[r * kRowWords + 9 + k]; }
  OG_D float* J1a_ptr(int r) { return rows + r * kRowWords + 3; }
  OG_D float* J2a_ptr(int r) { return rows + r * kRowWords + 9; }
  OG_D float& c(int r) { return rows[r * kRowWords + kRowC]; }
  OG_D float& cfm(int r) { return rows[r * kRowWords + kRowCfm]; }
  OG_D float& lo(int r) { return rows[r * kRowWords + kRowLo]; }
  OG_D float& hi(int r) { return rows[r * kRowWords + kRowHi]; }
  OG_D int& findex(int r) { return reinterpret_cast<int*>(rows)[r * kRowWords + kRowFindex]; }
  // findex of row r: row v of the same joint
  OG_D void set_findex(int r, int v) { findex(r) = fbase + v; }
};

// Body state a joint reads: placement, orientation and velocities.
struct BodyRef {
  float pos[3], q[4], R[12], lvel[3], avel[3];
};

OG_D void load_body_ref(const BatchDev& d, int gb, BodyRef& b) {
  const float4 p = d.pos[gb], q = d.q[gb], lv = d.lvel[gb], av = d.avel[gb];
  b.pos[0] = p.x; b.pos[1] = p.y; b.pos[2] = p.z;
  b.q[0] = q.x; b.q[1] = q.y; b.q[2] = q.z; b.q[3] = q.w;
  r_from_q(b.R, b.q);
  b.lvel[0] = lv.x; b.lvel[1] = lv.y; b.lvel[2] = lv.z;
  b.avel[0] = av.x; b.avel[1] = av.y; b.avel[2] = av.z;
}

// setBall (ode/src/joints/joint.cpp:85-128)
OG_D void set_ball(const BodyRef& B1, const BodyRef* B2, Info2& in, const float* anchor1,
                   const float* anchor2) {
  float a1[3], a2[3];
  in.J1l(0, 0) = 1.f; in.J1l(1, 1) = 1.f; in.J1l(2, 2) = 1.f;
  mul0_331(a1, B1.R, anchor1);
  // dSetCrossMatrixMinus
  in.J1a(0, 1) = +a1[2]; in.J1a(0, 2) = -a1[1];
  in.J1a(1, 0) = -a1[2]; in.J1a(1, 2) = +a1[0];
  in.J1a(2, 0) = +a1[1]; in.J1a(2, 1) = -a1[0];
  if (B2) {
    in.J2l(0, 0) = -1.f; in.J2l(1, 1) = -1.f; in.J2l(2, 2) = -1.f;
    mul0_331(a2, B2->R, anchor2);
    // dSetCrossMatrixPlus
    in.J2a(0, 1) = -a2[2]; in.J2a(0, 2) = +a2[1];
    in.J2a(1, 0) = +a2[2]; in.J2a(1, 2) = -a2[0];
    in.J2a(2, 0) = -a2[1]; in.J2a(2, 1) = +a2[0];
  }
  const float k = in.fps * in.erp;
  if (B2) {
    for (int j = 0; j < 3; j++) in.c(j) = k * (a2[j] + B2->pos[j] - a1[j] - B1.pos[j]);
  } else {
    for (int j = 0; j < 3; j++) in.c(j) = k * (anchor2[j] - a1[j] - B1.pos[j]);
  }
}

// setBall2 (ode/src/joints/joint.cpp:134-196)
OG_D void set_ball2(const BodyRef& B1, const BodyRef* B2, Info2& in, const float* anchor1,
                    const float* anchor2, const float* axis, float erp1) {
  float a1[3], a2[3], q1[3], q2[3];
  plane_space(axis, q1, q2);
  for (int i = 0; i < 3; i++) { in.J1l(0, i) = axis[i]; in.J1l(1, i) = q1[i]; in.J1l(2, i) = q2[i]; }
  mul0_331(a1, B1.R, anchor1);
  cross3(in.J1a_ptr(0), a1, axis);
  cross3(in.J1a_ptr(1), a1, q1);
  cross3(in.J1a_ptr(2), a1, q2);
  if (B2) {
    for (int i = 0; i < 3; i++) { in.J2l(0, i) = -axis[i]; in.J2l(1, i) = -q1[i]; in.J2l(2, i) = -q2[i]; }
    mul0_331(a2, B2->R, anchor2);
    const float* ax3[3] = {axis, q1, q2};
    for (int r = 0; r < 3; ++r) {
      float t[3];
      cross3(t, a2, ax3[r]);
      in.J2a(r, 0) = -t[0]; in.J2a(r, 1) = -t[1]; in.J2a(r, 2) = -t[2];
    }
  }
  const float k1 = in.fps * erp1;
  const float k = in.fps * in.erp;
  for (int i = 0; i < 3; i++) a1[i] += B1.pos[i];
  float d[3];
  if (B2) {
    for (int i = 0; i < 3; i++) a2[i] += B2->pos[i];
    d[0] = a2[0] - a1[0]; d[1] = a2[1] - a1[1]; d[2] = a2[2] - a1[2];
  } else {
    d[0] = anchor2[0] - a1[0]; d[1] = anchor2[1] - a1[1]; d[2] = anchor2[2] - a1[2];
  }
  in.c(0) = k1 * dot3(axis, d);
  in.c(1) = k * dot3(q1, d);
  in.c(2) = k * dot3(q2, d);
}

// getHingeAngleFromRelativeQuat (ode/src/joints/joint.cpp:381-420)
OG_D float hinge_angle_from_qrel(const float* qrel, const float* axis) {
  const float cost2 = qrel[0];
  const float sint2 = sqrtf(qrel[1] * qrel[1] + qrel[2] * qrel[2] + qrel[3] * qrel[3]);
  float theta = (dot3(qrel + 1, axis) >= 0.f) ? (2.f * atan2f(sint2, cost2))
                                               : (2.f * atan2f(sint2, -cost2));
  if ((double)theta > 3.14159265358979323846) theta -= (float)(2.0 * 3.14159265358979323846);
  return -theta;
}

// getHingeAngle (ode/src/joints/joint.cpp:432-450)
OG_D float hinge_angle(const BodyRef& B1, const BodyRef* B2, const DevJoint& J) {
  float qrel[4];
  if (B2) {
    float qq[4];
    qmul1(qq, B1.q, B2->q);
    qmul2(qrel, qq, J.qrel);
  } else {
    qmul3(qrel, B1.q, J.qrel);
  }
  return hinge_angle_from_qrel(qrel, J.axis1);
}

// dRFrom2Axes (ode/src/rotation.cpp:94-133): columns a, b orthogonalised
// against a, and a x b. A zero-length input leaves R as given.
OG_D void r_from_2axes(float* R, float ax, float ay, float az, float bx, float by, float bz) {
  float l = sqrtf(ax * ax + ay * ay + az * az);
  if (l <= 0.f) return;
  l = 1.0f / l;
  ax *= l; ay *= l; az *= l;
  const float k = ax * bx + ay * by + az * bz;
  bx -= k * ax; by -= k * ay; bz -= k * az;
  l = sqrtf(bx * bx + by * by + bz * bz);
  if (l <= 0.f) return;
  l = 1.0f / l;
  bx *= l; by *= l; bz *= l;
  R[0] = ax; R[4] = ay; R[8] = az;
  R[1] = bx; R[5] = by; R[9] = bz;
  R[2] = -by * az + ay * bz; R[6] = -bz * ax + az * bx; R[10] = -bx * ay + ax * by;
  R[3] = 0.f; R[7] = 0.f; R[11] = 0.f;
}

// dQfromR (ode/src/rotation.cpp:258-306)
OG_D void q_from_r(float* q, const float* R) {
  const float tr = R[0] + R[5] + R[10];
  float s;
  if (tr >= 0.f) {
    s = sqrtf(tr + 1.f);
    q[0] = 0.5f * s;
    s = 0.5f * (1.0f / s);
    q[1] = (R[9] - R[6]) * s; q[2] = (R[2] - R[8]) * s; q[3] = (R[4] - R[1]) * s;
    return;
  }
  int c;
  if (R[5] > R[0]) c = (R[10] > R[5]) ? 2 : 1;
  else c = (R[10] > R[0]) ? 2 : 0;
  if (c == 0) {
    s = sqrtf((R[0] - (R[5] + R[10])) + 1.f);
    q[1] = 0.5f * s;
    s = 0.5f * (1.0f / s);
    q[2] = (R[1] + R[4]) * s; q[3] = (R[8] + R[2]) * s; q[0] = (R[9] - R[6]) * s;
  } else if (c == 1) {
    s = sqrtf((R[5] - (R[10] + R[0])) + 1.f);
    q[2] = 0.5f * s;
    s = 0.5f * (1.0f / s);
    q[3] = (R[6] + R[9]) * s; q[1] = (R[1] + R[4]) * s; q[0] = (R[2] - R[8]) * s;
  } else {
    s = sqrtf((R[10] - (R[0] + R[5])) + 1.f);
    q[3] = 0.5f * s;
    s = 0.5f * (1.0f / s);
    q[1] = (R[8] + R[2]) * s; q[2] = (R[6] + R[9]) * s; q[0] = (R[4] - R[1]) * s;
  }
}

// dxJointUniversal::getAxes (ode/src/joints/universal.cpp:55-70)
OG_D void universal_axes(const BodyRef& B1, const BodyRef* B2, const DevJoint& J, float* ax1, float* ax2) {
  mul0_331(ax1, B1.R, J.axis1);
  if (B2) mul0_331(ax2, B2->R, J.axis2);
  else { ax2[0] = J.axis2[0]; ax2[1] = J.axis2[1]; ax2[2] = J.axis2[2]; }
}

// dxJointUniversal::getAngles (ode/src/joints/universal.cpp:73-167): angle 1
// from the cross frame dRFrom2Axes(ax1, ax2) against qrel1, angle 2 from that
// frame turned half a revolution about the bisector of ax1 and ax2 against qrel2.
OG_D void universal_angles(const BodyRef& B1, const BodyRef* B2, const DevJoint& J, float& angle1,
                           float& angle2) {
  float ax1[3], ax2[3], R[12], qcross[4], qq[4], qrel[4];
  universal_axes(B1, B2, J, ax1, ax2);
  for (int k = 0; k < 12; ++k) R[k] = (k % 5 == 0) ? 1.f : 0.f;
  r_from_2axes(R, ax1[0], ax1[1], ax1[2], ax2[0], ax2[1], ax2[2]);
  q_from_r(qcross, R);
  qmul1(qq, B1.q, qcross);
  qmul2(qrel, qq, J.qrel);
  angle1 = hinge_angle_from_qrel(qrel, J.axis1);
  qrel[0] = 0.f;
  qrel[1] = ax1[0] + ax2[0];
  qrel[2] = ax1[1] + ax2[1];
  qrel[3] = ax1[2] + ax2[2];
  const float l = 1.0f / sqrtf(qrel[1] * qrel[1] + qrel[2] * qrel[2] + qrel[3] * qrel[3]);
  qrel[1] *= l; qrel[2] *= l; qrel[3] *= l;
  float qcross2[4];
  qmul0(qcross2, qrel, qcross);
  if (B2) {
    qmul1(qq, B2->q, qcross2);
    qmul2(qrel, qq, J.qrel2);
  } else {
    qmul2(qrel, qcross2, J.qrel2);
  }
  angle2 = -hinge_angle_from_qrel(qrel, J.axis2);
}

// dJointGetSliderPosition (ode/src/joints/slider.cpp:42-79)
OG_D float slider_position(const BodyRef& B1, const BodyRef* B2, const DevJoint& J) {
  float ax1[3], q[3];
  mul0_331(ax1, B1.R, J.axis1);
  if (B2) {
    mul0_331(q, B2->R, J.offset);
    for (int i = 0; i < 3; ++i) q[i] = B1.pos[i] - q[i] - B2->pos[i];
  } else {
    for (int i = 0; i < 3; ++i) q[i] = B1.pos[i] - J.offset[i];
    if (J.reverse) { ax1[0] = -ax1[0]; ax1[1] = -ax1[1]; ax1[2] = -ax1[2]; }
  }
  return dot3(ax1, q);
}

// dxJointAMotor::computeGlobalAxes (ode/src/joints/amotor.cpp:52-94)
OG_D void amotor_axes(const BodyRef& B1, const BodyRef* B2, const DevJoint& J, float (&ax)[3][3]) {
  if (J.am_mode == AMOTOR_EULER) {
    mul0_331(ax[0], B1.R, J.am_axis[0]);
    if (B2) mul0_331(ax[2], B2->R, J.am_axis[2]);
    else { ax[2][0] = J.am_axis[2][0]; ax[2][1] = J.am_axis[2][1]; ax[2][2] = J.am_axis[2][2]; }
    cross3(ax[1], ax[2], ax[0]);
    safe_normalize3(ax[1]);
    return;
  }
  for (int i = 0; i < J.am_num; ++i) {
    if (J.am_rel[i] == 1) mul0_331(ax[i], B1.R, J.am_axis[i]);
    else if (J.am_rel[i] == 2) {
      if (B2) mul0_331(ax[i], B2->R, J.am_axis[i]);
    } else {
      ax[i][0] = J.am_axis[i][0]; ax[i][1] = J.am_axis[i][1]; ax[i][2] = J.am_axis[i][2];
    }
  }
}

// dxJointAMotor::computeEulerAngles (ode/src/joints/amotor.cpp:98-139)
OG_D void amotor_euler_angles(const BodyRef& B1, const BodyRef* B2, const DevJoint& J, const float (&ax)[3][3],
                              float* angle) {
  float ref1[3], ref2[3], q[3];
  mul0_331(ref1, B1.R, J.am_ref1);
  if (B2) mul0_331(ref2, B2->R, J.am_ref2);
  else { ref2[0] = J.am_ref2[0]; ref2[1] = J.am_ref2[1]; ref2[2] = J.am_ref2[2]; }
  cross3(q, ax[0], ref1);
  angle[0] = -atan2f(dot3(ax[2], q), dot3(ax[2], ref1));
  cross3(q, ax[0], ax[1]);
  angle[1] = -atan2f(dot3(ax[2], ax[0]), dot3(ax[2], q));
  cross3(q, ax[1], ax[2]);
  angle[2] = -atan2f(dot3(ref2, ax[1]), dot3(ref2, q));
}

// setFixedOrientation (ode/src/joints/joint.cpp:202-255): three rows from r0
// that hold the relative orientation at qrel, with info->erp as the joint
// finds it.
OG_D void set_fixed_orientation(const BodyRef& B1, const BodyRef* B2, Info2& in, const float* qrel, int r0) {
  in.J1a(r0, 0) = 1.f; in.J1a(r0 + 1, 1) = 1.f; in.J1a(r0 + 2, 2) = 1.f;
  if (B2) { in.J2a(r0, 0) = -1.f; in.J2a(r0 + 1, 1) = -1.f; in.J2a(r0 + 2, 2) = -1.f; }
  float qerr[4];
  if (B2) {
    float qq[4];
    qmul1(qq, B1.q, B2->q);
    qmul2(qerr, qq, qrel);
  } else {
    qmul3(qerr, B1.q, qrel);
  }
  if (qerr[0] < 0.f) { qerr[1] = -qerr[1]; qerr[2] = -qerr[2]; qerr[3] = -qerr[3]; }
  float e[3];
  mul0_331(e, B1.R, qerr + 1);
  const float k = in.fps * in.erp;
  in.c(r0) = 2.f * k * e[0];
  in.c(r0 + 1) = 2.f * k * e[1];
  in.c(r0 + 2) = 2.f * k * e[2];
}

// dxJointHinge2::measureAngle (ode/src/joints/hinge2.cpp:33-41)
OG_D float hinge2_angle(const BodyRef& B1, const BodyRef& B2, const DevJoint& J) {
  float a1[3], a2[3];
  mul0_331(a1, B2.R, J.axis2);
  mul1_331(a2, B1.R, a1);
  return -atan2f(dot3(J.v2, a2), dot3(J.v1, a2));
}

// dxJointLimitMotor::testRotationalLimit (ode/src/joints/joint.cpp:534-553)
OG_D int limot_test(const DevLimot& L, float angle, int& limit, float& err) {
  if (angle <= L.lostop) { limit = 1; err = angle - L.lostop; return 1; }
  if (angle >= L.histop) { limit = 2; err = angle - L.histop; return 1; }
  limit = 0;
  return 0;
}
OG_D bool limot_tested(const DevLimot& L) {
  return (L.lostop >= -kPi || L.histop <= kPi) && L.lostop <= L.histop;
}
// the slider's test (ode/src/joints/slider.cpp:150-151): any finite stop
OG_D bool limot_tested_linear(const DevLimot& L) {
  return (L.lostop > -INFINITY || L.histop < INFINITY) && L.lostop <= L.histop;
}

// Force and torques a powered-at-limit motor adds to the bodies, which the
// reference applies from inside getInfo2 via dBodyAddForce / dBodyAddTorque:
// body 1 gets f1 and t1, body 2 gets -f1 and t2.
struct LimotForce {
  float f1[3], t1[3], t2[3];
  int active;
};
OG_D LimotForce limot_force_none() { return LimotForce{{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, 0}; }

// dxJointLimitMotor::addLimot (ode/src/joints/joint.cpp:556-733). A linear
// limot (rotational = false) acts on J1l/J2l and, between two bodies, sets
// the angular parts to the torque-decoupling vector ltd = (x2 - x1)/2 x ax1.
OG_D int limot_add(const DevLimot& L, int limit, float limit_err, bool has_b2, const BodyRef& B1,
                   const BodyRef* B2, Info2& in, int row, const float* ax1, LimotForce& tq,
                   bool rotational = true) {
  int powered = L.fmax > 0.f;
  if (!(powered || limit)) return 0;
  float* J1 = rotational ? in.J1a_ptr(row) : &in.J1l(row, 0);
  float* J2 = rotational ? in.J2a_ptr(row) : &in.J2l(row, 0);
  J1[0] = ax1[0]; J1[1] = ax1[1]; J1[2] = ax1[2];
  if (has_b2) { J2[0] = -ax1[0]; J2[1] = -ax1[1]; J2[2] = -ax1[2]; }
  float ltd[3] = {0.f, 0.f, 0.f};
  if (!rotational && has_b2) {
    float c[3];
    c[0] = 0.5f * (B2->pos[0] - B1.pos[0]);
    c[1] = 0.5f * (B2->pos[1] - B1.pos[1]);
    c[2] = 0.5f * (B2->pos[2] - B1.pos[2]);
    cross3(ltd, c, ax1);
    for (int k = 0; k < 3; ++k) { in.J1a(row, k) = ltd[k]; in.J2a(row, k) = ltd[k]; }
  }
  if (limit && (L.lostop == L.histop)) powered = 0;
  if (powered) {
    in.cfm(row) = L.normal_cfm;
    if (!limit) {
      in.c(row) = L.vel;
      in.lo(row) = -L.fmax;
      in.hi(row) = L.fmax;
    } else {
      float fm = L.fmax;
      if ((L.vel > 0.f) || (L.vel == 0.f && limit == 2)) fm = -fm;
      if ((limit == 1 && L.vel > 0.f) || (limit == 2 && L.vel < 0.f)) fm *= L.fudge;
      // accumulated: an angular motor can meet limits on several axes
      if (rotational) {
        for (int k = 0; k < 3; ++k) { tq.t1[k] += -fm * ax1[k]; tq.t2[k] += fm * ax1[k]; }
      } else {
        for (int k = 0; k < 3; ++k) {
          tq.f1[k] += -fm * ax1[k];
          tq.t1[k] += has_b2 ? -fm * ltd[k] : 0.f;
          tq.t2[k] += -fm * ltd[k];
        }
      }
      tq.active = 1;
    }
  }
  if (limit) {
    const float k = in.fps * L.stop_erp;
    in.c(row) = -k * limit_err;
    in.cfm(row) = L.stop_cfm;
    if (L.lostop == L.histop) {
      in.lo(row) = -INFINITY; in.hi(row) = INFINITY;
    } else {
      if (limit == 1) { in.lo(row) = 0.f; in.hi(row) = INFINITY; }
      else { in.lo(row) = -INFINITY; in.hi(row) = 0.f; }
      if (L.bounce > 0.f) {
        float vel;
        if (rotational) {
          vel = dot3(B1.avel, ax1);
          if (B2) vel -= dot3(B2->avel, ax1);
        } else {
          vel = dot3(B1.lvel, ax1);
          if (B2) vel -= dot3(B2->lvel, ax1);
        }
        if (limit == 1) {
          if (vel < 0.f) { float nc = -L.bounce * vel; if (nc > in.c(row)) in.c(row) = nc; }
        } else {
          if (vel > 0.f) { float nc = -L.bounce * vel; if (nc < in.c(row)) in.c(row) = nc; }
        }
      }
    }
  }
  return 1;
}

// Per-joint state carried from getInfo1 to getInfo2 within a step.
struct JointInfo1 {
  int m;
  int limit1, limit2, limit3;
  float err1, err2, err3;
};

// getInfo1: contact (ode/src/joints/contact.cpp:47-71), ball (ball.cpp:56-60),
// hinge (hinge.cpp:54-74), slider (slider.cpp:134-167), universal
// (universal.cpp:265-293), hinge2 (hinge2.cpp:81-101), fixed (fixed.cpp:53-58).
// lm1: the joint's limot1 for this step (stops may differ from J.lm1).
OG_D JointInfo1 persistent_info1(const DevJoint& J, const DevLimot& lm1, const BodyRef& B1, const BodyRef* B2) {
  JointInfo1 r{0, 0, 0, 0, 0.f, 0.f, 0.f};
  switch (J.type) {
    case J_BALL: r.m = 3; break;
    case J_HINGE: {
      r.m = (lm1.fmax > 0.f) ? 6 : 5;
      if (limot_tested(lm1)) {
        if (limot_test(lm1, hinge_angle(B1, B2, J), r.limit1, r.err1)) r.m = 6;
      }
      break;
    }
    case J_HINGE2: {
      r.m = 4;
      if (limot_tested(lm1) && B2) limot_test(lm1, hinge2_angle(B1, *B2, J), r.limit1, r.err1);
      if (r.limit1 || lm1.fmax > 0.f) r.m++;
      if (J.lm2.fmax > 0.f) r.m++;
      break;
    }
    case J_SLIDER: {
      r.m = (lm1.fmax > 0.f) ? 6 : 5;
      if (limot_tested_linear(lm1)) {
        // the same comparisons as testRotationalLimit, on the slider position
        if (limot_test(lm1, slider_position(B1, B2, J), r.limit1, r.err1)) r.m = 6;
      }
      break;
    }
    case J_UNIVERSAL: {
      r.m = 4;
      const bool lim1 = limot_tested(lm1), lim2 = limot_tested(J.lm2);
      if (lim1 || lim2) {
        float a1, a2;
        universal_angles(B1, B2, J, a1, a2);
        if (lim1) limot_test(lm1, a1, r.limit1, r.err1);
        if (lim2) limot_test(J.lm2, a2, r.limit2, r.err2);
      }
      if (r.limit1 || lm1.fmax > 0.f) r.m++;
      if (r.limit2 || J.lm2.fmax > 0.f) r.m++;
      break;
    }
    case J_FIXED: r.m = 6; break;
    case J_AMOTOR: {
      // ode/src/joints/amotor.cpp:187-210: each axis's limit is tested every step
      float ang[3] = {J.am_angle[0], J.am_angle[1], J.am_angle[2]};
      if (J.am_mode == AMOTOR_EULER) {
        float ax[3][3];
        amotor_axes(B1, B2, J, ax);
        amotor_euler_angles(B1, B2, J, ax, ang);
      }
      const DevLimot* lm[3] = {&lm1, &J.lm2, &J.lm3};
      int* lim[3] = {&r.limit1, &r.limit2, &r.limit3};
      float* err[3] = {&r.err1, &r.err2, &r.err3};
      for (int i = 0; i < J.am_num; ++i)
        if (limot_test(*lm[i], ang[i], *lim[i], *err[i]) || lm[i]->fmax > 0.f) r.m++;
      break;
    }
    default: break;
  }
  return r;
}

OG_D int contact_info1(const DevSurface& S) {
  const float mu = S.mu < 0.f ? 0.f : S.mu;
  int m = 1;
  if (S.mode & SURF_MU2) {
    const float mu2 = S.mu2 < 0.f ? 0.f : S.mu2;
    if ((mu > 0.f) || (S.mu2 > 0.f)) m++;
    if (mu2 > 0.f) m++;
  } else {
    if (mu > 0.f) m += 2;
  }
  return m;
}

// dxJointContact::getInfo2 (ode/src/joints/contact.cpp:75-256)
OG_D void contact_info2(const DevContact& ct, const DevSurface& S, int the_m, const BodyRef& B1,
                        const BodyRef* B2, float min_depth, float max_vel, Info2& in) {
  const float mu = S.mu < 0.f ? 0.f : S.mu;
  const float mu2 = S.mu2 < 0.f ? 0.f : S.mu2;
  float normal[3];
  if (ct.reverse) { normal[0] = -ct.normal[0]; normal[1] = -ct.normal[1]; normal[2] = -ct.normal[2]; }
  else { normal[0] = ct.normal[0]; normal[1] = ct.normal[1]; normal[2] = ct.normal[2]; }
  float c1[3], c2[3] = {0.f, 0.f, 0.f};
  c1[0] = ct.pos[0] - B1.pos[0]; c1[1] = ct.pos[1] - B1.pos[1]; c1[2] = ct.pos[2] - B1.pos[2];
  in.J1l(0, 0) = normal[0]; in.J1l(0, 1) = normal[1]; in.J1l(0, 2) = normal[2];
  cross3(in.J1a_ptr(0), c1, normal);
  if (B2) {
    c2[0] = ct.pos[0] - B2->pos[0]; c2[1] = ct.pos[1] - B2->pos[1]; c2[2] = ct.pos[2] - B2->pos[2];
    in.J2l(0, 0) = -normal[0]; in.J2l(0, 1) = -normal[1]; in.J2l(0, 2) = -normal[2];
    float t[3];
    cross3(t, c2, normal);
    in.J2a(0, 0) = -t[0]; in.J2a(0, 1) = -t[1]; in.J2a(0, 2) = -t[2];
  }
  float erp = in.erp;
  if (S.mode & SURF_SOFT_ERP) erp = S.soft_erp;
  const float k = in.fps * erp;
  float depth = ct.depth - min_depth;
  if (depth < 0.f) depth = 0.f;
  if (S.mode & SURF_SOFT_CFM) in.cfm(0) = S.soft_cfm;
  float motionN = 0.f;
  if (S.mode & SURF_MOTIONN) motionN = S.motionN;
  float c0 = k * depth + motionN;
  if (c0 > max_vel) c0 = max_vel;
  if (S.mode & SURF_BOUNCE) {
    float outgoing = dot3(&in.J1l(0, 0), B1.lvel) + dot3(in.J1a_ptr(0), B1.avel);
    if (B2) outgoing += dot3(&in.J2l(0, 0), B2->lvel) + dot3(in.J2a_ptr(0), B2->avel);
    outgoing -= motionN;
    if (S.bounce_vel >= 0.f && (-outgoing) > S.bounce_vel) {
      const float newc = -S.bounce * outgoing + motionN;
      if (newc > c0) c0 = newc;
    }
  }
  in.c(0) = c0;
  in.lo(0) = 0.f;
  in.hi(0) = INFINITY;
  float t1[3], t2[3];
  if (the_m >= 2) {
    plane_space(normal, t1, t2);
    in.J1l(1, 0) = t1[0]; in.J1l(1, 1) = t1[1]; in.J1l(1, 2) = t1[2];
    cross3(in.J1a_ptr(1), c1, t1);
    if (B2) {
      in.J2l(1, 0) = -t1[0]; in.J2l(1, 1) = -t1[1]; in.J2l(1, 2) = -t1[2];
      float t[3];
      cross3(t, c2, t1);
      in.J2a(1, 0) = -t[0]; in.J2a(1, 1) = -t[1]; in.J2a(1, 2) = -t[2];
    }
    if (S.mode & SURF_MOTION1) in.c(1) = S.motion1;
    in.lo(1) = -mu;
    in.hi(1) = mu;
    if (S.mode & SURF_APPROX1_1) in.set_findex(1, 0);
    if (S.mode & SURF_SLIP1) in.cfm(1) = S.slip1;
  }
  if (the_m >= 3) {
    in.J1l(2, 0) = t2[0]; in.J1l(2, 1) = t2[1]; in.J1l(2, 2) = t2[2];
    cross3(in.J1a_ptr(2), c1, t2);
    if (B2) {
      in.J2l(2, 0) = -t2[0]; in.J2l(2, 1) = -t2[1]; in.J2l(2, 2) = -t2[2];
      float t[3];
      cross3(t, c2, t2);
      in.J2a(2, 0) = -t[0]; in.J2a(2, 1) = -t[1]; in.J2a(2, 2) = -t[2];
    }
    if (S.mode & SURF_MOTION2) in.c(2) = S.motion2;
    if (S.mode & SURF_MU2) { in.lo(2) = -mu2; in.hi(2) = mu2; }
    else { in.lo(2) = -mu; in.hi(2) = mu; }
    if (S.mode & SURF_APPROX1_2) in.set_findex(2, 0);
    if (S.mode & SURF_SLIP2) in.cfm(2) = S.slip2;
  }
}

// getInfo2 of the slider (slider.cpp:171-246), universal (universal.cpp:296-362)
// and fixed (fixed.cpp:62-105) joints; kept out of line so that the common
// joints' code does not carry their registers.
__device__ __noinline__ void persistent_info2_more(const DevJoint& J, const DevLimot& lm1, const JointInfo1& i1,
                                                   const BodyRef& B1, const BodyRef* B2, Info2& in,
                                                   LimotForce& tq1, LimotForce& tq2) {
  switch (J.type) {
    case J_SLIDER: {
      float c[3];
      if (B2) for (int i = 0; i < 3; ++i) c[i] = B2->pos[i] - B1.pos[i];
      set_fixed_orientation(B1, B2, in, J.qrel, 0);
      float ax1[3], p[3], q[3];
      mul0_331(ax1, B1.R, J.axis1);
      plane_space(ax1, p, q);
      if (B2) {
        float t[3];
        cross3(t, c, p);
        for (int i = 0; i < 3; ++i) { t[i] *= 0.5f; in.J1a(3, i) = t[i]; in.J2a(3, i) = t[i]; }
        cross3(t, c, q);
        for (int i = 0; i < 3; ++i) { t[i] *= 0.5f; in.J1a(4, i) = t[i]; in.J2a(4, i) = t[i]; }
        for (int i = 0; i < 3; ++i) { in.J2l(3, i) = -p[i]; in.J2l(4, i) = -q[i]; }
      }
      for (int i = 0; i < 3; ++i) { in.J1l(3, i) = p[i]; in.J1l(4, i) = q[i]; }
      const float k = in.fps * in.erp;
      if (B2) {
        float ofs[3];
        mul0_331(ofs, B2->R, J.offset);
        for (int i = 0; i < 3; ++i) c[i] += ofs[i];
        in.c(3) = k * dot3(p, c);
        in.c(4) = k * dot3(q, c);
      } else {
        float ofs[3];
        for (int i = 0; i < 3; ++i) ofs[i] = J.offset[i] - B1.pos[i];
        in.c(3) = k * dot3(p, ofs);
        in.c(4) = k * dot3(q, ofs);
        if (J.reverse) { ax1[0] = -ax1[0]; ax1[1] = -ax1[1]; ax1[2] = -ax1[2]; }
      }
      limot_add(lm1, i1.limit1, i1.err1, B2 != nullptr, B1, B2, in, 5, ax1, tq1, false);
      break;
    }
    case J_UNIVERSAL: {
      set_ball(B1, B2, in, J.anchor1, J.anchor2);
      float ax1[3], ax2[3], t[3], p[3];
      universal_axes(B1, B2, J, ax1, ax2);
      const float k = dot3(ax1, ax2);
      t[0] = ax2[0] - k * ax1[0];
      t[1] = ax2[1] - k * ax1[1];
      t[2] = ax2[2] - k * ax1[2];
      cross3(p, ax1, t);
      safe_normalize3(p);
      for (int i = 0; i < 3; ++i) in.J1a(3, i) = p[i];
      if (B2) for (int i = 0; i < 3; ++i) in.J2a(3, i) = -p[i];
      in.c(3) = in.fps * in.erp * -k;
      const int row = 4 + limot_add(lm1, i1.limit1, i1.err1, B2 != nullptr, B1, B2, in, 4, ax1, tq1);
      limot_add(J.lm2, i1.limit2, i1.err2, B2 != nullptr, B1, B2, in, row, ax2, tq2);
      break;
    }
    case J_AMOTOR: {
      // ode/src/joints/amotor.cpp:213-256: in Euler mode the rows constrain
      // w2 - w1 along ax1 x ax2, ax1 and ax0 x ax1
      float ax[3][3];
      amotor_axes(B1, B2, J, ax);
      float e0[3], e2[3];
      const float* axp[3] = {ax[0], ax[1], ax[2]};
      if (J.am_mode == AMOTOR_EULER) {
        cross3(e2, ax[0], ax[1]);
        axp[2] = e2;
        cross3(e0, ax[1], ax[2]);
        axp[0] = e0;
      }
      const DevLimot* lm[3] = {&lm1, &J.lm2, &J.lm3};
      const int lim[3] = {i1.limit1, i1.limit2, i1.limit3};
      const float err[3] = {i1.err1, i1.err2, i1.err3};
      int row = 0;
      for (int i = 0; i < J.am_num; ++i)
        row += limot_add(*lm[i], lim[i], err[i], B2 != nullptr, B1, B2, in, row, axp[i], i == 0 ? tq1 : tq2);
      break;
    }
    case J_FIXED: {
      // orientation rows with the erp the joint finds, then (like the ball
      // joint) info->erp = the joint's erp for the position rows and onwards
      set_fixed_orientation(B1, B2, in, J.qrel, 3);
      in.J1l(0, 0) = 1.f; in.J1l(1, 1) = 1.f; in.J1l(2, 2) = 1.f;
      in.erp = J.erp;
      in.cfm(0) = J.cfm; in.cfm(1) = J.cfm; in.cfm(2) = J.cfm;
      float ofs[3];
      mul0_331(ofs, B1.R, J.offset);
      if (B2) {
        // dSetCrossMatrixPlus
        in.J1a(0, 1) = -ofs[2]; in.J1a(0, 2) = +ofs[1];
        in.J1a(1, 0) = +ofs[2]; in.J1a(1, 2) = -ofs[0];
        in.J1a(2, 0) = -ofs[1]; in.J1a(2, 1) = +ofs[0];
        in.J2l(0, 0) = -1.f; in.J2l(1, 1) = -1.f; in.J2l(2, 2) = -1.f;
      }
      const float k = in.fps * in.erp;
      if (B2) {
        for (int j = 0; j < 3; ++j) in.c(j) = k * (B2->pos[j] - B1.pos[j] + ofs[j]);
      } else {
        for (int j = 0; j < 3; ++j) in.c(j) = k * (J.offset[j] - B1.pos[j]);
      }
      break;
    }
    default: break;
  }
}

// getInfo2 of the persistent joints: ball (ode/src/joints/ball.cpp:63-70),
// hinge (hinge.cpp:77-149), slider (slider.cpp:171-246), universal
// (universal.cpp:296-362), hinge2 (hinge2.cpp:109-180), fixed (fixed.cpp:62-105).
// The forces of up to two motors at a limit are returned in tq1/tq2 for the
// caller to apply.
OG_D void persistent_info2(const DevJoint& J, const DevLimot& lm1, const JointInfo1& i1, const BodyRef& B1,
                           const BodyRef* B2, Info2& in, LimotForce& tq1, LimotForce& tq2) {
  switch (J.type) {
    case J_BALL:
      // the reference writes info->erp here; the caller carries it forward
      in.erp = J.erp;
      in.cfm(0) = J.cfm; in.cfm(1) = J.cfm; in.cfm(2) = J.cfm;
      set_ball(B1, B2, in, J.anchor1, J.anchor2);
      break;
    case J_HINGE: {
      set_ball(B1, B2, in, J.anchor1, J.anchor2);
      float ax1[3], p[3], q[3];
      mul0_331(ax1, B1.R, J.axis1);
      plane_space(ax1, p, q);
      for (int k = 0; k < 3; ++k) { in.J1a(3, k) = p[k]; in.J1a(4, k) = q[k]; }
      if (B2) for (int k = 0; k < 3; ++k) { in.J2a(3, k) = -p[k]; in.J2a(4, k) = -q[k]; }
      float ax2[3], b[3];
      if (B2) mul0_331(ax2, B2->R, J.axis2);
      else { ax2[0] = J.axis2[0]; ax2[1] = J.axis2[1]; ax2[2] = J.axis2[2]; }
      cross3(b, ax1, ax2);
      const float k = in.fps * in.erp;
      in.c(3) = k * dot3(b, p);
      in.c(4) = k * dot3(b, q);
      limot_add(lm1, i1.limit1, i1.err1, B2 != nullptr, B1, B2, in, 5, ax1, tq1);
      break;
    }
    case J_HINGE2: {
      float ax1[3], ax2[3], q[3];
      mul0_331(ax1, B1.R, J.axis1);
      mul0_331(ax2, B2->R, J.axis2);
      cross3(q, ax1, ax2);
      const float sn = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
      const float cs = dot3(ax1, ax2);
      safe_normalize3(q);
      set_ball2(B1, B2, in, J.anchor1, J.anchor2, ax1, J.susp_erp);
      for (int k = 0; k < 3; ++k) in.J1a(3, k) = q[k];
      if (B2) for (int k = 0; k < 3; ++k) in.J2a(3, k) = -q[k];
      const float k = in.fps * in.erp;
      in.c(3) = k * (J.c0 * sn - J.s0 * cs);
      const int row = 4 + limot_add(lm1, i1.limit1, i1.err1, true, B1, B2, in, 4, ax1, tq1);
      limot_add(J.lm2, 0, 0.f, true, B1, B2, in, row, ax2, tq2);
      in.cfm(0) = J.susp_cfm;
      break;
    }
    case J_SLIDER:
    case J_UNIVERSAL:
    case J_FIXED:
    case J_AMOTOR: persistent_info2_more(J, lm1, i1, B1, B2, in, tq1, tq2); break;
    default: break;
  }
}

}  // namespace og
