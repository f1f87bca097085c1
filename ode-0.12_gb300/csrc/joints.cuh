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

// getHingeAngle (ode/src/joints/joint.cpp:381-451)
OG_D float hinge_angle(const BodyRef& B1, const BodyRef* B2, const DevJoint& J) {
  float qrel[4];
  if (B2) {
    float qq[4];
    qmul1(qq, B1.q, B2->q);
    qmul2(qrel, qq, J.qrel);
  } else {
    qmul3(qrel, B1.q, J.qrel);
  }
  const float cost2 = qrel[0];
  const float sint2 = sqrtf(qrel[1] * qrel[1] + qrel[2] * qrel[2] + qrel[3] * qrel[3]);
  float theta = (dot3(qrel + 1, J.axis1) >= 0.f) ? (2.f * atan2f(sint2, cost2))
                                                  : (2.f * atan2f(sint2, -cost2));
  if ((double)theta > 3.14159265358979323846) theta -= (float)(2.0 * 3.14159265358979323846);
  return -theta;
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

// Torque a powered-at-limit motor adds to body 1 (body 2 gets the negation),
// which the reference applies from inside getInfo2 via dBodyAddTorque.
struct LimotTorque {
  float t[3];
  int active;
};

// addLimot, rotational case (ode/src/joints/joint.cpp:556-733)
OG_D int limot_add(const DevLimot& L, int limit, float limit_err, bool has_b2, const BodyRef& B1,
                   const BodyRef* B2, Info2& in, int row, const float* ax1, LimotTorque& tq) {
  int powered = L.fmax > 0.f;
  if (!(powered || limit)) return 0;
  in.J1a(row, 0) = ax1[0]; in.J1a(row, 1) = ax1[1]; in.J1a(row, 2) = ax1[2];
  if (has_b2) { in.J2a(row, 0) = -ax1[0]; in.J2a(row, 1) = -ax1[1]; in.J2a(row, 2) = -ax1[2]; }
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
      tq.t[0] = -fm * ax1[0]; tq.t[1] = -fm * ax1[1]; tq.t[2] = -fm * ax1[2];
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
        float vel = dot3(B1.avel, ax1);
        if (B2) vel -= dot3(B2->avel, ax1);
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
  int limit1, limit2;
  float err1, err2;
};

// getInfo1: contact (ode/src/joints/contact.cpp:47-71), ball (ball.cpp:56-60),
// hinge (hinge.cpp:54-74), hinge2 (hinge2.cpp:81-101).
// lm1: the joint's limot1 for this step (stops may differ from J.lm1).
OG_D JointInfo1 persistent_info1(const DevJoint& J, const DevLimot& lm1, const BodyRef& B1, const BodyRef* B2) {
  JointInfo1 r{0, 0, 0, 0.f, 0.f};
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
    if (S.mode & SURF_APPROX1_1) in.findex(1) = 0;
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
    if (S.mode & SURF_APPROX1_2) in.findex(2) = 0;
    if (S.mode & SURF_SLIP2) in.cfm(2) = S.slip2;
  }
}

// getInfo2 of the persistent joints: ball (ode/src/joints/ball.cpp:63-70),
// hinge (hinge.cpp:77-149), hinge2 (hinge2.cpp:109-180). Up to two motor
// torques (body-1 sense) are returned in tq1/tq2 for the caller to apply.
OG_D void persistent_info2(const DevJoint& J, const DevLimot& lm1, const JointInfo1& i1, const BodyRef& B1,
                           const BodyRef* B2, Info2& in, LimotTorque& tq1, LimotTorque& tq2) {
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
    default: break;
  }
}

}  // namespace og
