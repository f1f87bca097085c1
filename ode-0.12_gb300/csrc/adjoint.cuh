// adjoint.cuh -- reverse-mode derivative of one batched world step.
//
// ODE has no gradients; this is the hand-written adjoint of the step the
// forward kernels run: controls (dJointAddHingeTorque / dJointAddHinge2Torques,
// body forces), the QuickStep prologue (quickstep.cpp:600-665), getInfo2 of
// ball and hinge joints and of contacts against planes, rhs / invM*J^T / Ad
// and the J, b scaling (quickstep.cpp:832-857, :117-136, :370-402), the
// SOR_LCP sweep with ODE's row order and reshuffles (quickstep.cpp:405-583)
// and the velocity / position / quaternion update (quickstep.cpp:905-916,
// util.cpp:255-360).
//
// One warp per world. The step's forward values come from the collide and
// setup kernels run again for that step (rows, invIw, accumulators, contacts,
// and the unscaled row dump with Ad and erp); the warp replays the SOR of the
// step in the forward's dependency-level schedule (ODE's order per body),
// recording lambda before every row update and which bound (if any) clamped
// it, then walks everything backwards, the sweep level by level in reverse. The
// clamp set is the one of the recorded sweep: a clamped row passes no
// derivative to its own lambda, and a friction row clamped by
// +-|hi * lambda[findex]| passes it to the normal row's lambda.
#pragma once
#include "world_solve.cuh"

namespace og {

// Status bits of the adjoint (per world): a part of the step whose
// derivative is not modelled was met (the gradient leaves it out).
enum {
  ADJ_UNSUPPORTED_JOINT = 1,     // a bouncing or motor-driven limit row, hinge2 without body 2,
                                 // slider, universal and fixed joints
  ADJ_UNSUPPORTED_CONTACT = 2,   // capsule vertex contact, geom under a field, bounce, fixed friction
                                 // direction
  ADJ_TOO_LARGE = 4,
  ADJ_PAIR_SWITCH = 8            // a body-body contact whose collider answer changes case within
                                 // every difference step
};

constexpr int kAdjBody = 48;   // per-body scratch words
constexpr int kAdjRow = 28;    // per-row scratch words
// body scratch: [0..2] d/dfacc [3..5] d/dtacc [6..14] d/dinvIw (3x3)
//               [15..23] d/dR (3x3) [24..29] d/dfc [30..35] fc [36..41] d/dtmp1
constexpr int kBF = 0, kBT = 3, kBIw = 6, kBR = 15, kBFcBar = 24, kBFc = 30, kBTmp1 = 36;
// row scratch: [0..11] d/dJ' (later d/dJ) [12..23] d/diMJ (later [12] d/dc)
//              [24] d/db' [25] d/d(Ad*cfm) [26] lambda [27] d/dlambda
constexpr int kRJ = 0, kRiMJ = 12, kRC = 12, kRb = 24, kRcfm = 25, kRLam = 26, kRLamBar = 27;

struct AdjDev {
  float* state_bar;          // [nb_total][13]: in d/d(state after), out d/d(state before)
  float* body_tmp;           // [nb_total][kAdjBody]
  float* row_tmp;            // [row_cap_total][kAdjRow]
  float* lam_tape;           // [row_cap_total * iters_max]
  unsigned char* code_tape;  // [row_cap_total * iters_max]
  uint16_t* seq_tape;        // [row_cap_total * rounds_max]
  const float* dbg;          // [row_cap_total][32] unscaled rows of the step
  float* g_jt;               // [n_ctrl][nj_total][2] accumulated, or null
  float* g_bf;               // [n_ctrl][nb_total][6] accumulated, or null
  int* status;               // [n_worlds] ADJ_* bits
  int iters_max, rounds_max;
};

// d/dq of R = dRfromQ(q) (ode/src/rotation.cpp:236-255) given d/dR (3x3).
OG_D void vjp_r_from_q(const float* q, const float* Rb, float* qb) {
  const float R00 = Rb[0], R01 = Rb[1], R02 = Rb[2], R10 = Rb[3], R11 = Rb[4], R12 = Rb[5];
  const float R20 = Rb[6], R21 = Rb[7], R22 = Rb[8];
  qb[0] += 2.f * (-q[3] * R01 + q[2] * R02 + q[3] * R10 - q[1] * R12 - q[2] * R20 + q[1] * R21);
  qb[1] += 2.f * (q[2] * R01 + q[3] * R02 + q[2] * R10 - 2.f * q[1] * R11 - q[0] * R12 + q[3] * R20 +
                  q[0] * R21 - 2.f * q[1] * R22);
  qb[2] += 2.f * (-2.f * q[2] * R00 + q[1] * R01 + q[0] * R02 + q[1] * R10 + q[3] * R12 - q[0] * R20 +
                  q[3] * R21 - 2.f * q[2] * R22);
  qb[3] += 2.f * (-2.f * q[3] * R00 - q[0] * R01 + q[1] * R02 + q[0] * R10 - 2.f * q[3] * R11 +
                  q[2] * R12 + q[1] * R20 + q[2] * R21);
}

// d/dn of (p, q) = dPlaneSpace(n) (ode/src/odemath.cpp:151-178), both branches.
OG_D void vjp_plane_space(const float* n, const float* pb, const float* qb, float* nb) {
  if (fabsf(n[2]) > kSqrt1_2) {
    // p = (0, -n2 k, n1 k), q = (a k, -n0 n1 k, -n0 n2 k), a = n1^2 + n2^2, k = a^-1/2
    const float a = n[1] * n[1] + n[2] * n[2];
    const float k = 1.0f / sqrtf(a), k3 = k * k * k;
    const float dk1 = -n[1] * k3, dk2 = -n[2] * k3;
    nb[1] += pb[1] * (-n[2] * dk1) + pb[2] * (k + n[1] * dk1);
    nb[2] += pb[1] * (-k - n[2] * dk2) + pb[2] * (n[1] * dk2);
    nb[1] += qb[0] * (n[1] * k);
    nb[2] += qb[0] * (n[2] * k);
    nb[0] += qb[1] * (-n[1] * k) + qb[2] * (-n[2] * k);
    nb[1] += qb[1] * (-n[0] * (k + n[1] * dk1)) + qb[2] * (-n[0] * n[2] * dk1);
    nb[2] += qb[1] * (-n[0] * n[1] * dk2) + qb[2] * (-n[0] * (k + n[2] * dk2));
  } else {
    // p = (-n1 k, n0 k, 0), q = (-n2 n0 k, -n2 n1 k, a k), a = n0^2 + n1^2
    const float a = n[0] * n[0] + n[1] * n[1];
    const float k = 1.0f / sqrtf(a), k3 = k * k * k;
    const float dk0 = -n[0] * k3, dk1 = -n[1] * k3;
    nb[0] += pb[0] * (-n[1] * dk0) + pb[1] * (k + n[0] * dk0);
    nb[1] += pb[0] * (-k - n[1] * dk1) + pb[1] * (n[0] * dk1);
    nb[0] += qb[2] * (n[0] * k);
    nb[1] += qb[2] * (n[1] * k);
    nb[2] += qb[0] * (-n[0] * k) + qb[1] * (-n[1] * k);
    nb[0] += qb[0] * (-n[2] * (k + n[0] * dk0)) + qb[1] * (-n[2] * n[1] * dk0);
    nb[1] += qb[0] * (-n[2] * n[0] * dk1) + qb[1] * (-n[2] * (k + n[1] * dk1));
  }
}

// M = R A R^T (3x4 R, 3x3 row-major A): Rb += Mb R A^T + Mb^T R A.
OG_D void vjp_rar(const float* R, const float* A, const float* Mb, float* Rb) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      float s = 0.f;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l)
          s += (Mb[i * 3 + k] * A[j * 3 + l] + Mb[k * 3 + i] * A[l * 3 + j]) * R[k * 4 + l];
      Rb[i * 3 + j] += s;
    }
}

// A chunk's row for this lane (idle lanes past the chunk's end load its last
// row again and are masked out): the row index and its eight 16-byte words.
OG_D bool adj_chunk_row(const float* rows, const SorSmem& S, unsigned c, int lane, int& r, float4 (&v)[8]) {
  const int last = (int)(c >> 11);
  const bool active = lane <= last;
  r = S.exec[(c & 0x7ffu) + (active ? lane : last)];
  const float4* src = reinterpret_cast<const float4*>(rows + (size_t)r * kRowWords);
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = src[k];
  return active;
}
OG_D void unpack_row_words(const float4 (&v)[8], float* J, float* iMJ, float& b, float& cfmA, float& lo, float& hi,
                           int& f, int& b1, int& b2) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    J[4 * k] = v[k].x; J[4 * k + 1] = v[k].y; J[4 * k + 2] = v[k].z; J[4 * k + 3] = v[k].w;
    iMJ[4 * k] = v[3 + k].x; iMJ[4 * k + 1] = v[3 + k].y; iMJ[4 * k + 2] = v[3 + k].z; iMJ[4 * k + 3] = v[3 + k].w;
  }
  b = v[6].x; cfmA = v[6].y; lo = v[6].z; hi = v[6].w;
  f = __float_as_int(v[7].x);
  b1 = __float_as_int(v[7].y);
  b2 = __float_as_int(v[7].z);
}

// One row update of the replayed sweep (the forward's arithmetic), recording
// lambda before the update and the bound that clamped it, if any.
OG_D void adj_replay_row(const float4 (&v)[8], int r, const SorSmem& S, float* lamT, unsigned char* codeT,
                         size_t tap) {
  float Jp[12], iMJ[12], bb, cfmA, lo, hi;
  int f, b1, b2;
  unpack_row_words(v, Jp, iMJ, bb, cfmA, lo, hi, f, b1, b2);
  float* fc1 = S.fc + 6 * b1;
  float* fc2 = S.fc + 6 * (b2 >= 0 ? b2 : kMaxB);
  const float old = S.lambda[r];
  lamT[tap + r] = old;
  float delta = bb - old * cfmA;
  delta -= (fc1[0] * Jp[0] + fc1[1] * Jp[1]) + (fc1[2] * Jp[2] + fc1[3] * Jp[3]) +
           (fc1[4] * Jp[4] + fc1[5] * Jp[5]);
  delta -= (fc2[0] * Jp[6] + fc2[1] * Jp[7]) + (fc2[2] * Jp[8] + fc2[3] * Jp[9]) +
           (fc2[4] * Jp[10] + fc2[5] * Jp[11]);
  float lo_act = lo, hi_act = hi;
  if (f >= 0) {
    hi_act = fabsf(hi * S.lambda[f]);
    lo_act = -hi_act;
  }
  const float nl = old + delta;
  unsigned char code = 0;
  float lam_new = nl;
  if (nl < lo_act) { code = 1; lam_new = lo_act; delta = lo_act - old; }
  else if (nl > hi_act) { code = 2; lam_new = hi_act; delta = hi_act - old; }
  codeT[tap + r] = code;
  S.lambda[r] = lam_new;
  for (int q = 0; q < 6; ++q) fc1[q] += delta * iMJ[q];
  if (b2 >= 0)
    for (int q = 0; q < 6; ++q) fc2[q] += delta * iMJ[6 + q];
}

// Derivative of the rows of persistent joint `ord` (rows r0..r0+m-1) with
// respect to its bodies' positions (into state_bar) and rotations (into the
// d/dR scratch).
// hinge2 (ode/src/joints/hinge2.cpp:109-180, setBall2 joint.cpp:134-196,
// measureAngle hinge2.cpp:33-41): d/d of its rows with respect to the bodies'
// positions and rotations. lm1: limot1 with this step's stops.
OG_D int vjp_hinge2(const BatchDev& d, const WorldDesc& D, const AdjDev& a, const DevJoint& J, const DevLimot& lm1,
                    int r0, int m, float k) {
  if (J.b2 < 0) return ADJ_UNSUPPORTED_JOINT;
  const int g1 = D.body_off + J.b1, g2 = D.body_off + J.b2;
  float R1[12], R2[12];
  body_R(d, g1, R1);
  body_R(d, g2, R2);
  const float4 x1 = d.pos[g1], x2 = d.pos[g2];
  float ax1[3], ax2[3], q1[3], q2[3], a1[3], a2[3];
  mul0_331(ax1, R1, J.axis1);
  mul0_331(ax2, R2, J.axis2);
  plane_space(ax1, q1, q2);
  mul0_331(a1, R1, J.anchor1);
  mul0_331(a2, R2, J.anchor2);
  const float dd[3] = {a2[0] + x2.x - a1[0] - x1.x, a2[1] + x2.y - a1[1] - x1.y, a2[2] + x2.z - a1[2] - x1.z};
  const float h1 = 1.0f / D.dt;
  const float kr[3] = {h1 * J.susp_erp, k, k};
  const float* dirs[3] = {ax1, q1, q2};
  const float* RT0 = a.row_tmp + (size_t)(D.row_off + r0) * kAdjRow;
  float ax1b[3] = {0.f, 0.f, 0.f}, ax2b[3] = {0.f, 0.f, 0.f}, q1b[3] = {0.f, 0.f, 0.f}, q2b[3] = {0.f, 0.f, 0.f};
  float a1b[3] = {0.f, 0.f, 0.f}, a2b[3] = {0.f, 0.f, 0.f}, db[3] = {0.f, 0.f, 0.f};
  float* dirb[3] = {ax1b, q1b, q2b};
  // rows 0..2: J1l = dir, J1a = a1 x dir, J2l = -dir, J2a = -(a2 x dir), c = k_r dir.d
  for (int r = 0; r < 3; ++r) {
    const float* t = RT0 + r * kAdjRow;
    const float* dir = dirs[r];
    float* dbar = dirb[r];
    float u[3];
    for (int i = 0; i < 3; ++i) dbar[i] += t[i] - t[6 + i];
    cross3(u, dir, t + 3);                 // d/da1 of a1 x dir
    for (int i = 0; i < 3; ++i) a1b[i] += u[i];
    cross3(u, t + 3, a1);                  // d/ddir of a1 x dir
    for (int i = 0; i < 3; ++i) dbar[i] += u[i];
    cross3(u, dir, t + 9);                 // J2a = -(a2 x dir)
    for (int i = 0; i < 3; ++i) a2b[i] -= u[i];
    cross3(u, t + 9, a2);
    for (int i = 0; i < 3; ++i) dbar[i] -= u[i];
    const float cb = kr[r] * t[kRC];
    for (int i = 0; i < 3; ++i) { dbar[i] += cb * dd[i]; db[i] += cb * dir[i]; }
  }
  vjp_plane_space(ax1, q1b, q2b, ax1b);
  // row 3: J1a = qn, J2a = -qn, c = k (c0 sn - s0 cs), q = ax1 x ax2, sn = |q|, cs = ax1.ax2
  {
    float q[3];
    cross3(q, ax1, ax2);
    const float sn = sqrtf(dot3(q, q));
    const float* t = RT0 + 3 * kAdjRow;
    if (sn > 0.f) {
      const float qn[3] = {q[0] / sn, q[1] / sn, q[2] / sn};
      float qnb[3];
      for (int i = 0; i < 3; ++i) qnb[i] = t[3 + i] - t[9 + i];
      const float snb = k * t[kRC] * J.c0;
      const float csb = -k * t[kRC] * J.s0;
      const float pr = dot3(qn, qnb);
      float qb[3];
      for (int i = 0; i < 3; ++i) qb[i] = snb * qn[i] + (qnb[i] - qn[i] * pr) / sn;
      float u[3];
      cross3(u, ax2, qb);
      for (int i = 0; i < 3; ++i) ax1b[i] += u[i] + csb * ax2[i];
      cross3(u, qb, ax1);
      for (int i = 0; i < 3; ++i) ax2b[i] += u[i] + csb * ax1[i];
    }
  }
  int flags = 0;
  // limot rows: limot1 about ax1 (row 4), limot2 about ax2 (next row)
  int row = 4;
  if (row < m) {
    // is row 4 limot1's? (it is when limot1 is limited or powered)
    BodyRef B1, B2;
    load_body_ref(d, g1, B1);
    load_body_ref(d, g2, B2);
    int limit = 0;
    float err = 0.f;
    if (limot_tested(lm1)) limot_test(lm1, hinge2_angle(B1, B2, J), limit, err);
    if (limit || lm1.fmax > 0.f) {
      const float* t = RT0 + row * kAdjRow;
      for (int i = 0; i < 3; ++i) ax1b[i] += t[3 + i] - t[9 + i];
      if (limit) {
        if (lm1.bounce > 0.f && lm1.lostop != lm1.histop) flags |= ADJ_UNSUPPORTED_JOINT;
        // c = -fps stop_erp (angle - stop); angle = -atan2(v2.b, v1.b), b = R1^T R2 axis2
        const float angb = -(h1 * lm1.stop_erp) * t[kRC];
        float e[3], bb[3];
        mul0_331(e, R2, J.axis2);
        mul1_331(bb, R1, e);
        const float y = dot3(J.v2, bb), x = dot3(J.v1, bb);
        const float r2 = x * x + y * y;
        if (r2 > 0.f) {
          const float yb = -angb * x / r2, xb = angb * y / r2;
          float bbar[3], ebar[3];
          for (int i = 0; i < 3; ++i) bbar[i] = yb * J.v2[i] + xb * J.v1[i];
          mul0_331(ebar, R1, bbar);
          float* Rb1 = a.body_tmp + (size_t)g1 * kAdjBody + kBR;
          float* Rb2 = a.body_tmp + (size_t)g2 * kAdjBody + kBR;
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
              atomicAdd(Rb1 + i * 3 + j, e[i] * bbar[j]);
              atomicAdd(Rb2 + i * 3 + j, ebar[i] * J.axis2[j]);
            }
        }
      }
      ++row;
    }
  }
  if (row < m) {
    const float* t = RT0 + row * kAdjRow;
    for (int i = 0; i < 3; ++i) ax2b[i] += t[3 + i] - t[9 + i];
  }
  // chain to the bodies
  for (int i = 0; i < 3; ++i) { a1b[i] -= db[i]; a2b[i] += db[i]; }
  float* xb1 = a.state_bar + (size_t)g1 * 13;
  float* xb2 = a.state_bar + (size_t)g2 * 13;
  for (int i = 0; i < 3; ++i) { atomicAdd(xb1 + i, -db[i]); atomicAdd(xb2 + i, db[i]); }
  float* Rb1 = a.body_tmp + (size_t)g1 * kAdjBody + kBR;
  float* Rb2 = a.body_tmp + (size_t)g2 * kAdjBody + kBR;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      atomicAdd(Rb1 + i * 3 + j, ax1b[i] * J.axis1[j] + a1b[i] * J.anchor1[j]);
      atomicAdd(Rb2 + i * 3 + j, ax2b[i] * J.axis2[j] + a2b[i] * J.anchor2[j]);
    }
  return flags;
}

// d/d(b, c) of a = f(b, c) for the bilinear quaternion products (qmul1:
// b* c, qmul2: b c*, qmul3: b* c*), given d/da: each partial is the product
// with a unit quaternion in that slot.
template <void (*F)(float*, const float*, const float*)>
OG_D void vjp_qmul(const float* qb_, const float* qc_, const float* ab, float* bb, float* cb) {
  for (int i = 0; i < 4; ++i) {
    float e[4] = {0.f, 0.f, 0.f, 0.f}, t[4];
    e[i] = 1.f;
    if (bb) { F(t, e, qc_); bb[i] += ab[0] * t[0] + ab[1] * t[1] + ab[2] * t[2] + ab[3] * t[3]; }
    if (cb) { F(t, qb_, e); cb[i] += ab[0] * t[0] + ab[1] * t[1] + ab[2] * t[2] + ab[3] * t[3]; }
  }
}

// d/dq1, d/dq2 of the hinge angle (getHingeAngle, ode/src/joints/joint.cpp:
// 381-450, as hinge_angle computes it from the bodies' quaternions) given its
// derivative angb. The angle is -2 atan2(|v|, +-w) of the relative rotation
// qrel = (q1* q2) qrel0* (w, v), the sign of w that of v . axis.
OG_D void vjp_hinge_angle(const BodyRef& B1, const BodyRef* B2, const DevJoint& J, float angb, float* q1b,
                          float* q2b) {
  float qq[4], qrel[4];
  if (B2) {
    qmul1(qq, B1.q, B2->q);
    qmul2(qrel, qq, J.qrel);
  } else {
    qmul3(qrel, B1.q, J.qrel);
  }
  const float* v = qrel + 1;
  const float sn = sqrtf(dot3(v, v));
  const float sgn = dot3(v, J.axis1) >= 0.f ? 1.f : -1.f;
  const float c = sgn * qrel[0];
  const float den = sn * sn + c * c;
  if (!(sn > 0.f) || !(den > 0.f)) return;
  const float thb = -angb;                          // angle = -theta
  float qrelb[4];
  qrelb[0] = thb * (-2.f * sn / den) * sgn;
  const float vs = thb * (2.f * c / den) / sn;
  qrelb[1] = vs * v[0]; qrelb[2] = vs * v[1]; qrelb[3] = vs * v[2];
  if (B2) {
    float qqb[4] = {0.f, 0.f, 0.f, 0.f};
    vjp_qmul<qmul2>(qq, J.qrel, qrelb, qqb, nullptr);
    vjp_qmul<qmul1>(B1.q, B2->q, qqb, q1b, q2b);
  } else {
    vjp_qmul<qmul3>(B1.q, J.qrel, qrelb, q1b, nullptr);
  }
}

OG_D int vjp_joint(const BatchDev& d, const WorldDesc& D, const AdjDev& a, int w, int ord, int r0, int m,
                   float k, const float* stops) {
  const DevJoint& J = d.joints[D.joint_off + ord];
  if (J.type == J_HINGE2) return vjp_hinge2(d, D, a, J, step_limot1(J, stops, ord), r0, m, k);
  if (J.type != J_BALL && J.type != J_HINGE) return ADJ_UNSUPPORTED_JOINT;
  int flags = 0;
  const int g1 = D.body_off + J.b1, g2 = J.b2 >= 0 ? D.body_off + J.b2 : -1;
  float R1[12], R2[12];
  body_R(d, g1, R1);
  if (g2 >= 0) body_R(d, g2, R2);
  float* xb1 = a.state_bar + (size_t)g1 * 13;
  float* xb2 = g2 >= 0 ? a.state_bar + (size_t)g2 * 13 : nullptr;
  float* Rb1 = a.body_tmp + (size_t)g1 * kAdjBody + kBR;
  float* Rb2 = g2 >= 0 ? a.body_tmp + (size_t)g2 * kAdjBody + kBR : nullptr;
  const float* RT0 = a.row_tmp + (size_t)(D.row_off + r0) * kAdjRow;
  // ball part, rows 0..2 (setBall, joint.cpp:85-128)
  float a1b[3] = {0.f, 0.f, 0.f}, a2b[3] = {0.f, 0.f, 0.f};
  for (int r = 0; r < 3; ++r) {
    const float* t = RT0 + r * kAdjRow;
    const float cb = t[kRC] * k;
    atomicAdd(xb1 + r, -cb);
    a1b[r] -= cb;
    if (g2 >= 0) { atomicAdd(xb2 + r, cb); a2b[r] += cb; }
  }
  {
    // J1a rows: (0, a1z, -a1y), (-a1z, 0, a1x), (a1y, -a1x, 0)
    const float* t0 = RT0 + 0 * kAdjRow + 3;
    const float* t1 = RT0 + 1 * kAdjRow + 3;
    const float* t2 = RT0 + 2 * kAdjRow + 3;
    a1b[0] += t1[2] - t2[1];
    a1b[1] += -t0[2] + t2[0];
    a1b[2] += t0[1] - t1[0];
    if (g2 >= 0) {
      const float* u0 = RT0 + 0 * kAdjRow + 9;
      const float* u1 = RT0 + 1 * kAdjRow + 9;
      const float* u2 = RT0 + 2 * kAdjRow + 9;
      a2b[0] += -u1[2] + u2[1];
      a2b[1] += u0[2] - u2[0];
      a2b[2] += -u0[1] + u1[0];
    }
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      atomicAdd(Rb1 + i * 3 + j, a1b[i] * J.anchor1[j]);
      if (g2 >= 0) atomicAdd(Rb2 + i * 3 + j, a2b[i] * J.anchor2[j]);
    }
  if (J.type == J_HINGE) {
    // rows 3, 4 (hinge.cpp:77-149) and the motor row 5
    float ax1[3], p[3], q[3], ax2[3], b[3];
    mul0_331(ax1, R1, J.axis1);
    plane_space(ax1, p, q);
    if (g2 >= 0) mul0_331(ax2, R2, J.axis2);
    else { ax2[0] = J.axis2[0]; ax2[1] = J.axis2[1]; ax2[2] = J.axis2[2]; }
    cross3(b, ax1, ax2);
    const float* t3 = RT0 + 3 * kAdjRow;
    const float* t4 = RT0 + 4 * kAdjRow;
    const float c3 = t3[kRC] * k, c4 = t4[kRC] * k;
    float pb[3], qb[3], bb[3], ax1b[3] = {0.f, 0.f, 0.f}, ax2b[3];
    for (int i = 0; i < 3; ++i) {
      pb[i] = t3[3 + i] + c3 * b[i];
      qb[i] = t4[3 + i] + c4 * b[i];
      if (g2 >= 0) { pb[i] -= t3[9 + i]; qb[i] -= t4[9 + i]; }
      bb[i] = c3 * p[i] + c4 * q[i];
    }
    // b = ax1 x ax2: d/dax1 = ax2 x bb, d/dax2 = bb x ax1
    cross3(ax1b, ax2, bb);
    cross3(ax2b, bb, ax1);
    vjp_plane_space(ax1, pb, qb, ax1b);
    if (m > 5) {
      const float* t5 = RT0 + 5 * kAdjRow;
      for (int i = 0; i < 3; ++i) ax1b[i] += t5[3 + i] - (g2 >= 0 ? t5[9 + i] : 0.f);
      // a motor row's rhs is the constant target velocity; a limit row's is
      // -fps stop_erp (angle - stop) (joint.cpp:556-733), through the hinge
      // angle into both quaternions
      const DevLimot lm1 = step_limot1(J, stops, ord);
      BodyRef B1, B2;
      load_body_ref(d, g1, B1);
      if (g2 >= 0) load_body_ref(d, g2, B2);
      int limit = 0;
      float err = 0.f;
      if (limot_tested(lm1)) limot_test(lm1, hinge_angle(B1, g2 >= 0 ? &B2 : nullptr, J), limit, err);
      if (limit) {
        // a bounce adds the relative velocity; a powered motor at the limit
        // adds torques to the bodies from inside getInfo2
        if (lm1.lostop != lm1.histop && (lm1.bounce > 0.f || lm1.fmax > 0.f)) flags |= ADJ_UNSUPPORTED_JOINT;
        float q1b[4] = {0.f, 0.f, 0.f, 0.f}, q2b[4] = {0.f, 0.f, 0.f, 0.f};
        vjp_hinge_angle(B1, g2 >= 0 ? &B2 : nullptr, J, -(lm1.stop_erp / D.dt) * t5[kRC], q1b, q2b);
        for (int i = 0; i < 4; ++i) {
          atomicAdd(xb1 + 3 + i, q1b[i]);
          if (g2 >= 0) atomicAdd(xb2 + 3 + i, q2b[i]);
        }
      }
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        atomicAdd(Rb1 + i * 3 + j, ax1b[i] * J.axis1[j]);
        if (g2 >= 0) atomicAdd(Rb2 + i * 3 + j, ax2b[i] * J.axis2[j]);
      }
  }
  return flags;
}

// Contact between two bodies (dCollide(g_i, g_k), body 1 = body(g_i)): the
// rows (contact.cpp:75-256: J1l = n, J1a = (pos - x1) x n, J2l = -n,
// J2a = -(pos - x2) x n, the friction rows along dPlaneSpace(n), the normal
// row's rhs k depth) are differentiated analytically with respect to the
// contact point, normal and depth and the two body positions; the contact
// point, normal and depth with respect to both bodies' positions and
// rotation matrices are the collider's Jacobian, taken by central
// differences of the same FP32 collider along the seven directions per body
// that a change of position and quaternion can take (three translations,
// three rotations, the scale of R). In each perturbed answer the contact is
// the nearest one with nearly the same normal; a step that crosses one of the
// collider's case boundaries (axis choice, clipping, culling, a shallow
// point's depth test) so that no such contact lies within 50 steps is
// retried at a quarter of its size, three times (down to 7.8e-6); a contact
// that vanishes on one side at every size takes the one-sided difference on
// the other, and is unsupported only when it vanishes on both.
constexpr float kPairStep = 5e-4f;
__device__ __noinline__ int vjp_contact_pair(const BatchDev& d, const WorldDesc& D, const AdjDev& a, int ci,
                                             int r0, int m, float erp_world) {
  const DevContact& ct = d.contacts[D.contact_off + ci];
  const DevSurface& S = d.surfaces[ct.surface];
  if (ct.geoms < 0 || ct.reverse || (S.mode & (SURF_BOUNCE | SURF_FDIR1)) || m == 2) return ADJ_UNSUPPORTED_CONTACT;
  const int pair = ct.geoms & 0xffff;
  const int gi = pair & 0xff, gk = (pair >> 8) & 0xff;
  if (d.gtype[D.geom_off + gi] == G_HEIGHTFIELD || d.gtype[D.geom_off + gk] == G_HEIGHTFIELD)
    return ADJ_UNSUPPORTED_CONTACT;
  if (d.gbody[D.geom_off + gi] != ct.b1 || d.gbody[D.geom_off + gk] != ct.b2) return ADJ_UNSUPPORTED_CONTACT;
  const int g1 = D.body_off + ct.b1, g2 = D.body_off + ct.b2;
  const float4 x14 = d.pos[g1], x24 = d.pos[g2];
  const float x1[3] = {x14.x, x14.y, x14.z}, x2[3] = {x24.x, x24.y, x24.z};
  const float* n = ct.normal;
  float t1[3], t2[3];
  plane_space(n, t1, t2);
  const float* dirs[3] = {n, t1, t2};
  const float c1[3] = {ct.pos[0] - x1[0], ct.pos[1] - x1[1], ct.pos[2] - x1[2]};
  const float c2[3] = {ct.pos[0] - x2[0], ct.pos[1] - x2[1], ct.pos[2] - x2[2]};
  const float* RT0 = a.row_tmp + (size_t)(D.row_off + r0) * kAdjRow;
  float dirb[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
  float c1b[3] = {0.f, 0.f, 0.f}, c2b[3] = {0.f, 0.f, 0.f};
  for (int r = 0; r < m; ++r) {
    const float* t = RT0 + r * kAdjRow;
    float u[3];
    for (int i = 0; i < 3; ++i) dirb[r][i] += t[i] - t[6 + i];
    cross3(u, t + 3, c1);                    // J1a = c1 x dir
    for (int i = 0; i < 3; ++i) dirb[r][i] += u[i];
    cross3(u, dirs[r], t + 3);
    for (int i = 0; i < 3; ++i) c1b[i] += u[i];
    cross3(u, t + 9, c2);                    // J2a = -(c2 x dir)
    for (int i = 0; i < 3; ++i) dirb[r][i] -= u[i];
    cross3(u, dirs[r], t + 9);
    for (int i = 0; i < 3; ++i) c2b[i] -= u[i];
  }
  float nb[3] = {dirb[0][0], dirb[0][1], dirb[0][2]};
  if (m == 3) vjp_plane_space(n, dirb[1], dirb[2], nb);
  float erp = erp_world;
  if (S.mode & SURF_SOFT_ERP) erp = S.soft_erp;
  const float kk = (1.0f / D.dt) * erp;
  const float dep = ct.depth - D.min_depth;
  const float motionN = (S.mode & SURF_MOTIONN) ? S.motionN : 0.f;
  const float depth_b = (dep > 0.f && kk * dep + motionN < D.max_vel) ? RT0[kRC] * kk : 0.f;
  const float posb[3] = {c1b[0] + c2b[0], c1b[1] + c2b[1], c1b[2] + c2b[2]};
  float* xb1 = a.state_bar + (size_t)g1 * 13;
  float* xb2 = a.state_bar + (size_t)g2 * 13;
  for (int i = 0; i < 3; ++i) { atomicAdd(xb1 + i, -c1b[i]); atomicAdd(xb2 + i, -c2b[i]); }
  // the collider's Jacobian by central differences, evaluated with body 1
  // at the origin (the colliders move with a common translation, and the
  // smaller coordinates carry less FP32 rounding); a step that changes the
  // contact count or jumps the contact is retried at a quarter of its size
  GeomView v0[2];
  geom_view(d, D, gi, v0[0]);
  geom_view(d, D, gk, v0[1]);
  for (int i = 0; i < 3; ++i) { v0[1].pos[i] -= v0[0].pos[i]; v0[0].pos[i] = 0.f; }
  const float pos_l[3] = {ct.pos[0] - x1[0], ct.pos[1] - x1[1], ct.pos[2] - x1[2]};
  Contact cc[8];
  float* Rb[2] = {a.body_tmp + (size_t)g1 * kAdjBody + kBR, a.body_tmp + (size_t)g2 * kAdjBody + kBR};
  float* xb[2] = {xb1, xb2};
  // per body: three translations, three small rotations about the world axes
  // (R -> (I + d [e_k]x) R) and a scale (R -> (1 + d) R): the directions a
  // change of the quaternion moves R in (dRfromQ of a non-unit q scales R)
  float gdir[2][7];
  // the contact in an answer of the collider: the nearest one with a normal
  // within a few degrees of this one's (another shallow contact of the pair
  // may come and go without changing this one); false when none lies within
  // `reach`
  auto match = [&](const GeomView* v, float reach, float* out) {
    const int nn = collide_primitive(v[0], v[1], (unsigned)D.max_contacts, cc);
    int best = -1;
    float bd = reach * reach;
    for (int j = 0; j < nn; ++j) {
      const float dx = cc[j].pos[0] - pos_l[0], dy = cc[j].pos[1] - pos_l[1], dz = cc[j].pos[2] - pos_l[2];
      const float d2 = dx * dx + dy * dy + dz * dz;
      if (d2 <= bd && dot3(cc[j].normal, n) > 0.99f) { bd = d2; best = j; }
    }
    if (best < 0) return false;
    for (int i = 0; i < 3; ++i) { out[i] = cc[best].pos[i]; out[3 + i] = cc[best].normal[i]; }
    out[6] = cc[best].depth;
    return true;
  };
  float fbase[7];
  if (!match(v0, 1e-4f, fbase)) return ADJ_PAIR_SWITCH;
  for (int k = 0; k < 14; ++k) {
    const int side = k / 7, e = k % 7;
    // one direction's derivative: central differences at the first step of
    // 5e-4, 1.25e-4, 3.1e-5, 7.8e-6 where the contact is found on both sides;
    // failing that (a contact within a step of vanishing), the one-sided
    // difference on the side where it is found at 1.25e-4
    float f[2][7];
    bool have[2] = {false, false};
    float step = kPairStep, used = 0.f;
    int mode = 0;   // 1 central, 2 plus side only, 3 minus side only
    for (int attempt = 0; attempt < 4 && !mode; ++attempt, step *= 0.25f) {
      for (int sg = 0; sg < 2; ++sg) {
        GeomView v[2] = {v0[0], v0[1]};
        const float delta = sg ? -step : step;
        float* R = v[side].R;
        if (e < 3) {
          v[side].pos[e] += delta;
        } else if (e < 6) {
          float w[3] = {0.f, 0.f, 0.f};
          w[e - 3] = delta;
          for (int j = 0; j < 3; ++j) {
            const float col[3] = {R[j], R[4 + j], R[8 + j]};
            float u[3];
            cross3(u, w, col);
            R[j] = col[0] + u[0]; R[4 + j] = col[1] + u[1]; R[8 + j] = col[2] + u[2];
          }
        } else {
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) R[i * 4 + j] *= 1.f + delta;
        }
        have[sg] = match(v, 50.f * step, f[sg]);
      }
      if (have[0] && have[1]) { mode = 1; used = step; }
      else if (attempt == 1 && (have[0] || have[1])) { mode = have[0] ? 2 : 3; used = step; }
    }
    if (!mode) return ADJ_PAIR_SWITCH;
    float dfd[7];
    for (int i = 0; i < 7; ++i)
      dfd[i] = mode == 1 ? (f[0][i] - f[1][i]) * (0.5f / used)
                         : mode == 2 ? (f[0][i] - fbase[i]) / used : (fbase[i] - f[1][i]) / used;
    float g = depth_b * dfd[6];
    for (int i = 0; i < 3; ++i) g += posb[i] * dfd[i] + nb[i] * dfd[3 + i];
    gdir[side][e] = g;
  }
  // back to d/dx and d/dR: d/dR = sum_k g_k / (2 s^2) [e_k]x R + g_scale / (3 s^2) R,
  // s^2 = |R|^2 / 3 (the directions are orthogonal with these norms)
  for (int side = 0; side < 2; ++side) {
    const float* R = v0[side].R;
    float n2 = 0.f;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) n2 += R[i * 4 + j] * R[i * 4 + j];
    if (!(n2 > 0.f)) return ADJ_UNSUPPORTED_CONTACT;
    const float cr = 1.5f / n2, cs = gdir[side][6] / n2;
    const float w[3] = {cr * gdir[side][3], cr * gdir[side][4], cr * gdir[side][5]};
    for (int i = 0; i < 3; ++i) atomicAdd(xb[side] + i, gdir[side][i]);
    for (int j = 0; j < 3; ++j) {
      const float col[3] = {R[j], R[4 + j], R[8 + j]};
      float u[3];
      cross3(u, w, col);
      for (int i = 0; i < 3; ++i) atomicAdd(Rb[side] + i * 3 + j, u[i] + cs * col[i]);
    }
  }
  return 0;
}

// Derivative of a contact's rows with respect to the contact point and depth,
// and of those (sphere / box / capsule against a plane) with respect to the
// body's position and rotation.
OG_D int vjp_contact(const BatchDev& d, const WorldDesc& D, const AdjDev& a, int ci, int r0, int m,
                     float erp_world) {
  const DevContact& ct = d.contacts[D.contact_off + ci];
  const DevSurface& S = d.surfaces[ct.surface];
  if (ct.b2 >= 0) return vjp_contact_pair(d, D, a, ci, r0, m, erp_world);
  if (ct.geoms < 0) return ADJ_UNSUPPORTED_CONTACT;
  const int gA = D.geom_off + (ct.geoms & 0xff), gB = D.geom_off + ((ct.geoms >> 8) & 0xff);
  const unsigned kind = ((unsigned)ct.geoms >> 16) & 3u;
  int gp, gs;
  bool hf = false;
  if (d.gtype[gA] == G_PLANE || d.gtype[gA] == G_HEIGHTFIELD) { gp = gA; gs = gB; hf = d.gtype[gA] == G_HEIGHTFIELD; }
  else if (d.gtype[gB] == G_PLANE || d.gtype[gB] == G_HEIGHTFIELD) {
    gp = gB; gs = gA; hf = d.gtype[gB] == G_HEIGHTFIELD;
  }
  else return ADJ_UNSUPPORTED_CONTACT;
  if (hf && kind == kHFUnder) return ADJ_UNSUPPORTED_CONTACT;
  const int ts = d.gtype[gs];
  if (d.gbody[gs] != ct.b1 || (ts != 0 && ts != 1 && ts != 2)) return ADJ_UNSUPPORTED_CONTACT;
  if (S.mode & SURF_BOUNCE) return ADJ_UNSUPPORTED_CONTACT;
  const int g1 = D.body_off + ct.b1;
  const float4 x4 = d.pos[g1];
  const float x[3] = {x4.x, x4.y, x4.z};
  float R[12];
  body_R(d, g1, R);
  float normal[3];
  const float sg = ct.reverse ? -1.f : 1.f;
  for (int i = 0; i < 3; ++i) normal[i] = sg * ct.normal[i];
  float t1[3], t2[3];
  plane_space(normal, t1, t2);
  const float* dirs[3] = {normal, t1, t2};
  const float* RT0 = a.row_tmp + (size_t)(D.row_off + r0) * kAdjRow;
  // c1 = pos - x1; J1a(r) = c1 x dir_r  ->  d/dc1 += dir_r x d/dJ1a(r)
  float c1b[3] = {0.f, 0.f, 0.f};
  for (int r = 0; r < m; ++r) {
    float t[3];
    cross3(t, dirs[r], RT0 + r * kAdjRow + 3);
    c1b[0] += t[0]; c1b[1] += t[1]; c1b[2] += t[2];
  }
  // normal row rhs: c = min(k * max(depth - min_depth, 0) + motionN, max_vel)
  float erp = erp_world;
  if (S.mode & SURF_SOFT_ERP) erp = S.soft_erp;
  const float kk = (1.0f / D.dt) * erp;
  const float dep = ct.depth - D.min_depth;
  const float motionN = (S.mode & SURF_MOTIONN) ? S.motionN : 0.f;
  float depth_b = 0.f;
  if (dep > 0.f && kk * dep + motionN < D.max_vel) depth_b = RT0[kRC] * kk;
  // contact point and depth of the body-side geom against the plane; for a
  // heightfield's plane pass, the plane of the triangle (its upward normal
  // is the collider's normal, negated when the field came first)
  float np[3];
  if (hf) {
    const float sgn = (gp == gA) ? -1.f : 1.f;
    for (int i = 0; i < 3; ++i) np[i] = sgn * ct.normal[i];
  } else {
    const float4 pp = d.gparam[gp];
    np[0] = pp.x; np[1] = pp.y; np[2] = pp.z;
  }
  const float4 gprm = d.gparam[gs];
  if (hf && kind == kHFVertex) {
    // vertex pass: the contact point is a field sample (fixed); the depth is
    // the geom's point depth at it (dGeomSpherePointDepth / dGeomBoxPointDepth)
    float* xb = a.state_bar + (size_t)g1 * 13;
    float* Rb = a.body_tmp + (size_t)g1 * kAdjBody + kBR;
    for (int i = 0; i < 3; ++i) atomicAdd(xb + i, -c1b[i]);       // c1 = pos - x1
    if (depth_b == 0.f) return 0;
    const float v[3] = {ct.pos[0] - x[0], ct.pos[1] - x[1], ct.pos[2] - x[2]};
    if (ts == 0) {
      const float l = sqrtf(dot3(v, v));
      if (l > 0.f)
        for (int i = 0; i < 3; ++i) atomicAdd(xb + i, depth_b * v[i] / l);
      return 0;
    }
    if (ts != 1) return ADJ_UNSUPPORTED_CONTACT;
    float qv[3];
    mul1_331(qv, R, v);
    const float hs[3] = {0.5f * gprm.x, 0.5f * gprm.y, 0.5f * gprm.z};
    float dist[6];
    bool inside = true;
    for (int i = 0; i < 3; ++i) {
      dist[i] = hs[i] - qv[i];
      dist[i + 3] = hs[i] + qv[i];
      if (dist[i] < 0.f || dist[i + 3] < 0.f) inside = false;
    }
    int best = 0;
    for (int i = 1; i < 6; ++i)
      if (inside ? (dist[i] < dist[best]) : (dist[i] > dist[best])) best = i;
    // depth = +-dist[best]; dist = h -+ q_j, q = R^T (v - x)
    const int j = best % 3;
    const float dq = (inside ? 1.f : -1.f) * (best < 3 ? -1.f : 1.f) * depth_b;   // d/dq_j
    for (int i = 0; i < 3; ++i) {
      atomicAdd(xb + i, -dq * R[i * 4 + j]);
      atomicAdd(Rb + i * 3 + j, dq * v[i]);
    }
    return 0;
  }
  float s[3] = {0.f, 0.f, 0.f};
  float rad = 0.f;
  const float rel[3] = {ct.pos[0] - x[0], ct.pos[1] - x[1], ct.pos[2] - x[2]};
  if (ts == 0) {
    rad = gprm.x;
  } else if (ts == 1) {
    float sl[3];
    mul1_331(sl, R, rel);
    const float hs[3] = {0.5f * gprm.x, 0.5f * gprm.y, 0.5f * gprm.z};
    for (int i = 0; i < 3; ++i) s[i] = sl[i] >= 0.f ? hs[i] : -hs[i];
  } else {
    rad = gprm.x;
    const float cr[3] = {rel[0] + rad * np[0], rel[1] + rad * np[1], rel[2] + rad * np[2]};
    float sl[3];
    mul1_331(sl, R, cr);
    s[2] = sl[2] >= 0.f ? 0.5f * gprm.y : -0.5f * gprm.y;
  }
  // pos = x + R s - rad n ; depth = rad + d - n.(x + R s)
  float pb[3], gx[3];
  for (int i = 0; i < 3; ++i) { pb[i] = c1b[i]; gx[i] = pb[i] - depth_b * np[i]; }
  float* xb = a.state_bar + (size_t)g1 * 13;
  for (int i = 0; i < 3; ++i) atomicAdd(xb + i, gx[i] - c1b[i]);   // c1 = pos - x1
  float* Rb = a.body_tmp + (size_t)g1 * kAdjBody + kBR;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) atomicAdd(Rb + i * 3 + j, gx[i] * s[j]);
  return 0;
}

// Shared memory of one warp: the forward SOR layout, plus d/dfc and d/dlambda.
constexpr int kAdjSmemPerWarp = align16(kSorSmemPerWarp + (kMaxB + 1) * 6 * 4 + (kMaxR + 4) * 4);
static_assert(kAdjSmemPerWarp % 16 == 0, "per-warp slices must stay aligned");

OG_D void atomic_add3(float* p, const float* v) {
  atomicAdd(p + 0, v[0]); atomicAdd(p + 1, v[1]); atomicAdd(p + 2, v[2]);
}

// Shuffle of every island's order for round `round` (ODE's reshuffle at
// iteration 8 * round; islands draw from the RNG stream in island order).
OG_D void adj_shuffle(const int* rstart, int nisl, int n_shuffles, int round, unsigned seed, uint16_t* seq,
                      int lane) {
  unsigned prefix = 0;
  for (int ib = 0; ib < nisl; ib += 32) {
    const int isl = ib + lane;
    int m = 0;
    if (isl < nisl) m = rstart[isl + 1] - rstart[isl];
    const int draws = m > 0 ? n_shuffles * (m - 1) : 0;
    const int incl = warp_incl_scan(draws, lane);
    if (isl < nisl && m > 1) {
      unsigned s = lcg_jump(seed, prefix + (unsigned)(incl - draws) + (unsigned)(round * (m - 1)));
      uint16_t* sq = seq + rstart[isl];
      for (int q = 1; q < m; ++q) {
        s = lcg_next(s);
        const int sw = rand_int_from(s, q + 1);
        const uint16_t t = sq[q];
        sq[q] = sq[sw];
        sq[sw] = t;
      }
    }
    prefix += (unsigned)__shfl_sync(kFull, incl, 31);
  }
  __syncwarp();
}

// One row of the sweep backwards: the row's state before its update in the
// replayed sweep (lambda from the tape, fc by undoing the update), the
// derivative through the update's clamp case, accumulated into the row's
// record, d/dlambda and d/dfc.
OG_D void adj_reverse_row(const float4 (&v)[8], int r, float old, unsigned char code, const SorSmem& S, float* fcb,
                          float* lamb, float* rt0) {
  float Jp[12], iMJ[12], bb, cfmA, lo, hi;
  int f, b1, b2;
  unpack_row_words(v, Jp, iMJ, bb, cfmA, lo, hi, f, b1, b2);
  float4* rt4 = reinterpret_cast<float4*>(rt0 + r * kAdjRow);   // 112-byte records, 16-byte aligned
  float acc[kAdjRow];
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    const float4 t = rt4[q];
    acc[4 * q] = t.x; acc[4 * q + 1] = t.y; acc[4 * q + 2] = t.z; acc[4 * q + 3] = t.w;
  }
  const float dl = S.lambda[r] - old;
  float* fc1 = S.fc + 6 * b1;
  float* fb1 = fcb + 6 * b1;
  float* fc2 = b2 >= 0 ? S.fc + 6 * b2 : nullptr;
  float* fb2 = b2 >= 0 ? fcb + 6 * b2 : nullptr;
  // fc before the update
  for (int q = 0; q < 6; ++q) fc1[q] -= dl * iMJ[q];
  if (fc2) for (int q = 0; q < 6; ++q) fc2[q] -= dl * iMJ[6 + q];
  float dlb = 0.f;
  for (int q = 0; q < 6; ++q) { dlb += iMJ[q] * fb1[q]; acc[kRiMJ + q] += dl * fb1[q]; }
  if (fc2)
    for (int q = 0; q < 6; ++q) { dlb += iMJ[6 + q] * fb2[q]; acc[kRiMJ + 6 + q] += dl * fb2[q]; }
  const float lnb = lamb[r] + dlb;
  float oldb = -dlb;
  float ub = 0.f;
  if (code == 0) {
    ub = lnb;
  } else if (f >= 0) {
    const float lf = S.lambda[f];
    const float dbound = (hi * lf >= 0.f) ? hi : -hi;   // d|hi lf| / dlf
    lamb[f] += (code == 2 ? lnb : -lnb) * dbound;
  }
  // u = old + b' - old cfmA - J'.fc
  oldb += ub * (1.f - cfmA);
  acc[kRb] += ub;
  acc[kRcfm] -= ub * old;
  for (int q = 0; q < 6; ++q) { acc[kRJ + q] -= ub * fc1[q]; fb1[q] -= ub * Jp[q]; }
  if (fc2)
    for (int q = 0; q < 6; ++q) { acc[kRJ + 6 + q] -= ub * fc2[q]; fb2[q] -= ub * Jp[6 + q]; }
#pragma unroll
  for (int q = 0; q < 7; ++q)
    rt4[q] = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
  lamb[r] = oldb;
  S.lambda[r] = old;
}

// One warp per world: the adjoint of one step (see the file comment).
__global__ void __launch_bounds__(128, 1) adjoint_step_kernel(BatchDev d, AdjDev a, int step) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w >= d.n_worlds) return;
  unsigned char* base = smem_raw + (size_t)(threadIdx.x >> 5) * kAdjSmemPerWarp;
  const SorSmem S = carve_sor(base);
  float* fcb = reinterpret_cast<float*>(base + kSorSmemPerWarp);      // [(kMaxB+1)*6] d/dfc
  float* lamb = fcb + (kMaxB + 1) * 6;                                // [kMaxR+4] d/dlambda
  const WorldDesc D = d.world[w];
  if (D.nb > kMaxB || D.iterations > a.iters_max) {
    if (lane == 0) a.status[w] |= ADJ_TOO_LARGE;
    return;
  }
  const float h = D.dt, h1 = 1.0f / D.dt;
  const int M = d.nrows[w], nisl = d.nislands[w];
  const int iters = D.iterations, rc = D.row_cap;
  const int n_shuffles = (iters + 7) / 8;
  const int* rstart = d.island_rstart + D.body_off + w;
  const float* rows = d.rows + (size_t)D.row_off * kRowWords;
  const float* dbg = a.dbg + (size_t)D.row_off * kRowWords;
  float* bt0 = a.body_tmp + (size_t)D.body_off * kAdjBody;
  float* rt0 = a.row_tmp + (size_t)D.row_off * kAdjRow;
  float* lamT = a.lam_tape + (size_t)D.row_off * a.iters_max;
  unsigned char* codeT = a.code_tape + (size_t)D.row_off * a.iters_max;
  uint16_t* seqT = a.seq_tape + (size_t)D.row_off * a.rounds_max;
  const unsigned seed = d.seed[w];
  int flags = 0;
  for (int i = lane; i < D.nb * kAdjBody; i += 32) bt0[i] = 0.f;
  for (int i = lane; i < M * kAdjRow; i += 32) rt0[i] = 0.f;
  for (int i = lane; i < (kMaxB + 1) * 6; i += 32) { S.fc[i] = 0.f; fcb[i] = 0.f; }
  for (int i = lane; i < kMaxR + 4; i += 32) { S.lambda[i] = 0.f; lamb[i] = 0.f; }
  __syncwarp();

  // 1. SOR replay with tape, in the forward's level schedule
  if (M > 0) {
    for (int isl = 0; isl < nisl; ++isl) {
      const int rs = rstart[isl], re = rstart[isl + 1];
      int negc = 0;
      for (int b0 = rs; b0 < re; b0 += 32) {
        const int r = b0 + lane;
        bool neg = false;
        if (r < re) neg = __float_as_int(rows[(size_t)r * kRowWords + kRowFindex]) == -1;
        const unsigned bal = __ballot_sync(kFull, neg && r < re);
        const int negb = negc + __popc(bal & ((1u << lane) - 1u));
        if (r < re) S.seq[neg ? rs + negb : re - 1 - ((r - rs) - negb)] = (uint16_t)r;
        negc += __popc(bal);
      }
    }
    __syncwarp();
    int nchunk = 0;
    for (int it = 0; it < iters; ++it) {
      if ((it & 7) == 0) {
        adj_shuffle(rstart, nisl, n_shuffles, it >> 3, seed, S.seq, lane);
        for (int i = lane; i < M; i += 32) seqT[(size_t)(it >> 3) * rc + i] = S.seq[i];
        nchunk = sor_schedule(rows, D.nb, S, M, lane);
      }
      // the next chunk's rows are loaded while a chunk updates (two register
      // buffers used in turn)
      const size_t tap = (size_t)it * rc;
      float4 va[8], vb[8];
      int ra = 0, rb = 0;
      bool aa = nchunk > 0 && adj_chunk_row(rows, S, S.chunk[0], lane, ra, va), ab = false;
      for (int k = 0; k < nchunk; k += 2) {
        if (k + 1 < nchunk) ab = adj_chunk_row(rows, S, S.chunk[k + 1], lane, rb, vb);
        if (aa) adj_replay_row(va, ra, S, lamT, codeT, tap);
        __syncwarp();
        if (k + 1 >= nchunk) break;
        if (k + 2 < nchunk) aa = adj_chunk_row(rows, S, S.chunk[k + 2], lane, ra, va);
        if (ab) adj_replay_row(vb, rb, S, lamT, codeT, tap);
        __syncwarp();
      }
    }
  }

  // 2. integration backwards (state_bar: after -> partial before)
  for (int b = lane; b < D.nb; b += 32) {
    const int gb = D.body_off + b;
    float* bt = bt0 + b * kAdjBody;
    float* sb = a.state_bar + (size_t)gb * 13;
    const float4 av4 = d.avel[gb], q4 = d.q[gb], t4 = d.tacc[gb];
    const float* fc = S.fc + 6 * b;
    const float* iw = d.invIw + 12 * gb;
    const float im = d.invMass[gb];
    float t3[3] = {h * t4.x, h * t4.y, h * t4.z}, r3[3];
    mul0_331(r3, iw, t3);
    float wn[3] = {av4.x, av4.y, av4.z};
    if (M > 0) { wn[0] += h * fc[3]; wn[1] += h * fc[4]; wn[2] += h * fc[5]; }
    wn[0] += r3[0]; wn[1] += r3[1]; wn[2] += r3[2];
    const float q[4] = {q4.x, q4.y, q4.z, q4.w};
    float qt[4];
    qt[0] = q[0] + h * 0.5f * (-wn[0] * q[1] - wn[1] * q[2] - wn[2] * q[3]);
    qt[1] = q[1] + h * 0.5f * (wn[0] * q[0] + wn[1] * q[3] - wn[2] * q[2]);
    qt[2] = q[2] + h * 0.5f * (-wn[0] * q[3] + wn[1] * q[0] + wn[2] * q[1]);
    qt[3] = q[3] + h * 0.5f * (wn[0] * q[2] - wn[1] * q[1] + wn[2] * q[0]);
    const float l2 = qt[0] * qt[0] + qt[1] * qt[1] + qt[2] * qt[2] + qt[3] * qt[3];
    const float il = 1.0f / sqrtf(l2);
    const float qn[4] = {qt[0] * il, qt[1] * il, qt[2] * il, qt[3] * il};
    const float qnb[4] = {sb[3], sb[4], sb[5], sb[6]};
    const float pr = qn[0] * qnb[0] + qn[1] * qnb[1] + qn[2] * qnb[2] + qn[3] * qnb[3];
    float qtb[4];
    for (int i = 0; i < 4; ++i) qtb[i] = il * (qnb[i] - qn[i] * pr);
    // qt = q + (h/2) G(wn) q
    const float hh = 0.5f * h;
    float qb[4];
    qb[0] = qtb[0] + hh * (wn[0] * qtb[1] + wn[1] * qtb[2] + wn[2] * qtb[3]);
    qb[1] = qtb[1] + hh * (-wn[0] * qtb[0] + wn[2] * qtb[2] - wn[1] * qtb[3]);
    qb[2] = qtb[2] + hh * (-wn[1] * qtb[0] - wn[2] * qtb[1] + wn[0] * qtb[3]);
    qb[3] = qtb[3] + hh * (-wn[2] * qtb[0] + wn[1] * qtb[1] - wn[0] * qtb[2]);
    float wb[3];
    wb[0] = sb[10] + hh * (-q[1] * qtb[0] + q[0] * qtb[1] - q[3] * qtb[2] + q[2] * qtb[3]);
    wb[1] = sb[11] + hh * (-q[2] * qtb[0] + q[3] * qtb[1] + q[0] * qtb[2] - q[1] * qtb[3]);
    wb[2] = sb[12] + hh * (-q[3] * qtb[0] - q[2] * qtb[1] + q[1] * qtb[2] + q[0] * qtb[3]);
    // pos' = pos + h v'
    const float xb[3] = {sb[0], sb[1], sb[2]};
    const float vb[3] = {sb[7] + h * xb[0], sb[8] + h * xb[1], sb[9] + h * xb[2]};
    // v' = v + h fc_l + h invM facc ; w' = w + h fc_a + invIw (h tacc)
    for (int i = 0; i < 3; ++i) {
      fcb[6 * b + i] = h * vb[i];
      fcb[6 * b + 3 + i] = h * wb[i];
      bt[kBF + i] = h * im * vb[i];
    }
    float tb[3];
    mul1_331(tb, iw, wb);
    const float tacc[3] = {t4.x, t4.y, t4.z};
    for (int i = 0; i < 3; ++i) {
      bt[kBT + i] = h * tb[i];
      for (int j = 0; j < 3; ++j) bt[kBIw + i * 3 + j] += h * wb[i] * tacc[j];
    }
    sb[3] = qb[0]; sb[4] = qb[1]; sb[5] = qb[2]; sb[6] = qb[3];
    sb[7] = vb[0]; sb[8] = vb[1]; sb[9] = vb[2];
    sb[10] = wb[0]; sb[11] = wb[1]; sb[12] = wb[2];
  }
  __syncwarp();

  if (M > 0) {
    // 3. SOR backwards: iterations in reverse, each round's levels in reverse
    int nchunk = 0;
    for (int it = iters - 1; it >= 0; --it) {
      if (it == iters - 1 || ((it + 1) & 7) == 0) {
        for (int i = lane; i < M; i += 32) S.seq[i] = seqT[(size_t)(it >> 3) * rc + i];
        __syncwarp();
        nchunk = sor_schedule(rows, D.nb, S, M, lane);
      }
      // the next chunk's rows and tape entries are loaded while a chunk is
      // reversed (two register buffers used in turn)
      const size_t tap = (size_t)it * rc;
      float4 va[8], vb[8];
      int ra = 0, rb = 0;
      float oa = 0.f, ob = 0.f;
      unsigned char ca = 0, cb = 0;
      bool aa = false, ab = false;
      if (nchunk > 0) {
        aa = adj_chunk_row(rows, S, S.chunk[nchunk - 1], lane, ra, va);
        oa = lamT[tap + ra];
        ca = codeT[tap + ra];
      }
      for (int k = nchunk - 1; k >= 0; k -= 2) {
        if (k - 1 >= 0) {
          ab = adj_chunk_row(rows, S, S.chunk[k - 1], lane, rb, vb);
          ob = lamT[tap + rb];
          cb = codeT[tap + rb];
        }
        if (aa) adj_reverse_row(va, ra, oa, ca, S, fcb, lamb, rt0);
        __syncwarp();
        if (k - 1 < 0) break;
        if (k - 2 >= 0) {
          aa = adj_chunk_row(rows, S, S.chunk[k - 2], lane, ra, va);
          oa = lamT[tap + ra];
          ca = codeT[tap + ra];
        }
        if (ab) adj_reverse_row(vb, rb, ob, cb, S, fcb, lamb, rt0);
        __syncwarp();
      }
    }

    // 4. row setup backwards: J' = Ad J, b' = Ad rhs, cfmA = Ad cfm', Ad = w / (J.iMJ + cfm'),
    //    iMJ = invM J, rhs = c / h - J.tmp1
    for (int r = lane; r < M; r += 32) {
      const float* dr = dbg + (size_t)r * kRowWords;
      const float* row = rows + (size_t)r * kRowWords;
      float* rt = rt0 + r * kAdjRow;
      const int b1 = __float_as_int(dr[kRowB1]), b2 = __float_as_int(dr[kRowB2]);
      const int nj = b2 >= 0 ? 12 : 6;
      const float Ad = dr[kDbgAd], rhs = dr[kRowC], cfmp = dr[kRowCfm];
      float J[12], iMJ[12], Jb[12], iMJb[12];
      for (int q = 0; q < 12; ++q) { J[q] = dr[q]; iMJ[q] = row[12 + q]; iMJb[q] = rt[kRiMJ + q]; }
      float Adb = rt[kRb] * rhs + rt[kRcfm] * cfmp;
      for (int q = 0; q < nj; ++q) Adb += rt[kRJ + q] * J[q];
      for (int q = 0; q < 12; ++q) Jb[q] = Ad * rt[kRJ + q];
      const float rhsb = Ad * rt[kRb];
      const float sbar = -Adb * Ad * Ad / D.sor_w;
      for (int q = 0; q < nj; ++q) { Jb[q] += sbar * iMJ[q]; iMJb[q] += sbar * J[q]; }
      const int bodies[2] = {b1, b2};
      for (int s2 = 0; s2 < (b2 >= 0 ? 2 : 1); ++s2) {
        const int gb = D.body_off + bodies[s2];
        float* bt = bt0 + bodies[s2] * kAdjBody;
        const float* iw = d.invIw + 12 * gb;
        const float im = d.invMass[gb];
        const int o = 6 * s2;
        for (int q = 0; q < 3; ++q) Jb[o + q] += im * iMJb[o + q];
        float t[3];
        mul1_331(t, iw, iMJb + o + 3);
        for (int q = 0; q < 3; ++q) Jb[o + 3 + q] += t[q];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) atomicAdd(bt + kBIw + i * 3 + j, iMJb[o + 3 + i] * J[o + 3 + j]);
        // tmp1 of the body
        const float4 f4 = d.facc[gb], t4 = d.tacc[gb], lv = d.lvel[gb], av = d.avel[gb];
        float tmp1[6];
        tmp1[0] = f4.x * im + lv.x * h1; tmp1[1] = f4.y * im + lv.y * h1; tmp1[2] = f4.z * im + lv.z * h1;
        const float tt[3] = {t4.x, t4.y, t4.z};
        float r3[3];
        mul0_331(r3, iw, tt);
        tmp1[3] = r3[0] + av.x * h1; tmp1[4] = r3[1] + av.y * h1; tmp1[5] = r3[2] + av.z * h1;
        for (int q = 0; q < 6; ++q) {
          Jb[o + q] -= rhsb * tmp1[q];
          atomicAdd(bt + kBTmp1 + q, -rhsb * J[o + q]);
        }
      }
      for (int q = 0; q < 12; ++q) rt[kRJ + q] = Jb[q];
      rt[kRC] = rhsb * h1;
    }
    __syncwarp();

    // 5. joint and contact rows backwards; the lane owning a joint's first row
    //    handles the joint (its rows are contiguous)
    const int njt_all = d.world[d.n_worlds - 1].joint_off + d.world[d.n_worlds - 1].njp;
    const float* stops = (d.joint_stop && d.n_ctrl_steps > 0)
                             ? d.joint_stop + (size_t)(step % d.n_ctrl_steps) * njt_all + D.joint_off
                             : nullptr;
    for (int r0 = lane; r0 < M; r0 += 32) {
      const int ord = __float_as_int(dbg[(size_t)r0 * kRowWords + kRowJoint]);
      if (r0 > 0 && __float_as_int(dbg[(size_t)(r0 - 1) * kRowWords + kRowJoint]) == ord) continue;
      int r1 = r0 + 1;
      while (r1 < M && __float_as_int(dbg[(size_t)r1 * kRowWords + kRowJoint]) == ord) ++r1;
      const float erp = dbg[(size_t)r0 * kRowWords + kDbgErp];
      if (ord < D.njp) flags |= vjp_joint(d, D, a, w, ord, r0, r1 - r0, h1 * erp, stops);
      else flags |= vjp_contact(d, D, a, ord - D.njp, r0, r1 - r0, erp);
    }
    __syncwarp();
  }

  // 6. tmp1 = [facc invM + v / h ; invIw tacc + w / h] backwards, and the prologue
  for (int b = lane; b < D.nb; b += 32) {
    const int gb = D.body_off + b;
    float* bt = bt0 + b * kAdjBody;
    float* sb = a.state_bar + (size_t)gb * 13;
    const float* iw = d.invIw + 12 * gb;
    const float im = d.invMass[gb];
    const float4 t4 = d.tacc[gb], av = d.avel[gb];
    const float tacc[3] = {t4.x, t4.y, t4.z};
    for (int q = 0; q < 3; ++q) {
      bt[kBF + q] += im * bt[kBTmp1 + q];
      sb[7 + q] += h1 * bt[kBTmp1 + q];
      sb[10 + q] += h1 * bt[kBTmp1 + 3 + q];
    }
    {
      float t[3];
      mul1_331(t, iw, bt + kBTmp1 + 3);
      for (int q = 0; q < 3; ++q) bt[kBT + q] += t[q];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) bt[kBIw + i * 3 + j] += bt[kBTmp1 + 3 + i] * tacc[j];
    }
    float R[12];
    body_R(d, gb, R);
    // invIw = R invI R^T
    vjp_rar(R, d.invI + 9 * gb, bt + kBIw, bt + kBR);
    // gyroscopic term: tacc -= w x (Iw w), Iw = R I R^T
    if (d.bflags[gb] & BODY_GYROSCOPIC) {
      float Ib[12], tmp[12], Iw[12];
      const float* ii = d.I + 9 * gb;
      for (int r = 0; r < 3; ++r) {
        Ib[r * 4 + 0] = ii[r * 3 + 0]; Ib[r * 4 + 1] = ii[r * 3 + 1];
        Ib[r * 4 + 2] = ii[r * 3 + 2]; Ib[r * 4 + 3] = 0.f;
      }
      mul2_333(tmp, Ib, R);
      mul0_333(Iw, R, tmp);
      const float w3[3] = {av.x, av.y, av.z};
      float y[3];
      mul0_331(y, Iw, w3);
      const float gb3[3] = {-bt[kBT + 0], -bt[kBT + 1], -bt[kBT + 2]};
      float t[3], yb[3];
      cross3(t, y, gb3);
      cross3(yb, gb3, w3);
      float u[3];
      mul1_331(u, Iw, yb);
      for (int q = 0; q < 3; ++q) sb[10 + q] += t[q] + u[q];
      float Iwb[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Iwb[i * 3 + j] = yb[i] * w3[j];
      vjp_rar(R, ii, Iwb, bt + kBR);
    }
  }
  __syncwarp();

  // 7. controls backwards
  const int nbt = d.world[d.n_worlds - 1].body_off + d.world[d.n_worlds - 1].nb;
  const int njt = d.world[d.n_worlds - 1].joint_off + d.world[d.n_worlds - 1].njp;
  const int cs = d.n_ctrl_steps > 0 ? step % d.n_ctrl_steps : 0;
  if (a.g_bf && d.n_ctrl_steps > 0)
    for (int b = lane; b < D.nb; b += 32) {
      float* g = a.g_bf + ((size_t)cs * nbt + D.body_off + b) * 6;
      const float* bt = bt0 + b * kAdjBody;
      for (int q = 0; q < 3; ++q) { g[q] += bt[kBF + q]; g[3 + q] += bt[kBT + q]; }
    }
  if (d.joint_torque && d.n_ctrl_steps > 0)
    for (int j = lane; j < D.njp; j += 32) {
      const DevJoint& J = d.joints[D.joint_off + j];
      const float* tq = d.joint_torque + ((size_t)cs * njt + D.joint_off + j) * 2;
      float* g = a.g_jt ? a.g_jt + ((size_t)cs * njt + D.joint_off + j) * 2 : nullptr;
      const float* tb1 = bt0 + J.b1 * kAdjBody + kBT;
      float tb[3] = {tb1[0], tb1[1], tb1[2]};
      if (J.b2 >= 0) {
        const float* tb2 = bt0 + J.b2 * kAdjBody + kBT;
        tb[0] -= tb2[0]; tb[1] -= tb2[1]; tb[2] -= tb2[2];
      }
      if (J.type == J_HINGE) {
        float R[12], ax[3];
        body_R(d, D.body_off + J.b1, R);
        mul0_331(ax, R, J.axis1);
        const float sgn = J.reverse ? -1.f : 1.f;
        if (g) g[0] += sgn * dot3(ax, tb);
        float* Rb = bt0 + J.b1 * kAdjBody + kBR;
        const float torque = sgn * tq[0];
        for (int i = 0; i < 3; ++i)
          for (int k = 0; k < 3; ++k) atomicAdd(Rb + i * 3 + k, torque * tb[i] * J.axis1[k]);
      } else if (J.type == J_HINGE2 && J.b2 >= 0) {
        float R1[12], R2[12], a1[3], a2[3];
        body_R(d, D.body_off + J.b1, R1);
        body_R(d, D.body_off + J.b2, R2);
        mul0_331(a1, R1, J.axis1);
        mul0_331(a2, R2, J.axis2);
        if (g) { g[0] += dot3(a1, tb); g[1] += dot3(a2, tb); }
        float* Rb1 = bt0 + J.b1 * kAdjBody + kBR;
        float* Rb2 = bt0 + J.b2 * kAdjBody + kBR;
        for (int i = 0; i < 3; ++i)
          for (int k = 0; k < 3; ++k) {
            atomicAdd(Rb1 + i * 3 + k, tq[0] * tb[i] * J.axis1[k]);
            atomicAdd(Rb2 + i * 3 + k, tq[1] * tb[i] * J.axis2[k]);
          }
      }
    }
  __syncwarp();

  // 8. rotations -> quaternions
  for (int b = lane; b < D.nb; b += 32) {
    const int gb = D.body_off + b;
    const float4 q4 = d.q[gb];
    const float q[4] = {q4.x, q4.y, q4.z, q4.w};
    vjp_r_from_q(q, bt0 + b * kAdjBody + kBR, a.state_bar + (size_t)gb * 13 + 3);
  }
  flags = __reduce_or_sync(kFull, flags);
  if (flags && lane == 0) a.status[w] |= flags;
}

}  // namespace og
