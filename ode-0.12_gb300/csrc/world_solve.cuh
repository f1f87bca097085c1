// world_solve.cuh -- phases 2 and 4-7 of a world step (see world_step.cuh).
#pragma once
#include "world_step.cuh"
#include "sor.cuh"
#include "sor_fwd.cuh"

namespace og {

// Phase 2 (quickstep.cpp:600-665): world-frame inverse inertia, gyroscopic
// torque and gravity of one body (global index gb).
OG_D void body_prologue(const BatchDev& d, const WorldDesc& D, int gb) {
  float R[12], tmp[12], invIb[12], invIw[12];
  body_R(d, gb, R);
  const float* ib = d.invI + 9 * gb;
  for (int r = 0; r < 3; ++r) {
    invIb[r * 4 + 0] = ib[r * 3 + 0]; invIb[r * 4 + 1] = ib[r * 3 + 1];
    invIb[r * 4 + 2] = ib[r * 3 + 2]; invIb[r * 4 + 3] = 0.f;
  }
  mul2_333(tmp, invIb, R);
  mul0_333(invIw, R, tmp);
  float* out = d.invIw + 12 * gb;
  for (int k = 0; k < 12; ++k) out[k] = invIw[k];
  float4 t = d.tacc[gb];
  const float4 av = d.avel[gb];
  if (d.bflags[gb] & BODY_GYROSCOPIC) {
    float Ib[12], Iw[12], t3[3], cr[3];
    const float* ii = d.I + 9 * gb;
    for (int r = 0; r < 3; ++r) {
      Ib[r * 4 + 0] = ii[r * 3 + 0]; Ib[r * 4 + 1] = ii[r * 3 + 1];
      Ib[r * 4 + 2] = ii[r * 3 + 2]; Ib[r * 4 + 3] = 0.f;
    }
    mul2_333(tmp, Ib, R);
    mul0_333(Iw, R, tmp);
    const float w3[3] = {av.x, av.y, av.z};
    mul0_331(t3, Iw, w3);
    cross3(cr, w3, t3);
    t.x = t.x - cr[0]; t.y = t.y - cr[1]; t.z = t.z - cr[2];
    d.tacc[gb] = t;
  }
  if (!(d.bflags[gb] & BODY_NO_GRAVITY)) {
    float4 f = d.facc[gb];
    const float m = d.mass[gb];
    if (D.gravity[0] != 0.f) f.x += m * D.gravity[0];
    if (D.gravity[1] != 0.f) f.y += m * D.gravity[1];
    if (D.gravity[2] != 0.f) f.z += m * D.gravity[2];
    d.facc[gb] = f;
  }
}
OG_D void phase_body_prologue(const BatchDev& d, const WorldDesc& D, int lane) {
  for (int b = lane; b < D.nb; b += 32) body_prologue(d, D, D.body_off + b);
}

// the step's row of per-joint stops (dJointSet*Param lo/hi stop before the step), or null
OG_D const float* step_stops(const BatchDev& d, const WorldDesc& D, int step) {
  const int njt = d.world[d.n_worlds - 1].joint_off + d.world[d.n_worlds - 1].njp;
  return (d.joint_stop && d.n_ctrl_steps > 0) ? d.joint_stop + (size_t)(step % d.n_ctrl_steps) * njt + D.joint_off
                                               : nullptr;
}

// limot1 as getInfo sees it this step: the stored one with the step's stops
// (when given) in place of lostop / histop.
OG_D DevLimot step_limot1(const DevJoint& J, const float* stops, int ord) {
  DevLimot L = J.lm1;
  if (stops && (J.type == J_HINGE || J.type == J_HINGE2 || J.type == J_SLIDER || J.type == J_UNIVERSAL ||
                J.type == J_AMOTOR)) {
    const float v = stops[ord];
    if (!isnan(v)) { L.lostop = v; L.histop = v; }
  }
  return L;
}

// getInfo2 of one joint (ordinal ord: persistent joints first, then
// contacts) into its m rows starting at world row r0, with the erp it meets
// (quickstep.cpp:763-830): rows cleared to the stepper's defaults, the
// joint's rows, powered-at-limit motor forces added to the bodies, and findex
// rebased to world rows.
OG_D void assemble_joint_rows(const BatchDev& d, const WorldDesc& D, int ord, int r0, int m, float erp,
                              const float* stops, float* dbg_rows) {
  const float h1 = 1.0f / D.dt;
  float* rows = d.rows + (size_t)(D.row_off + r0) * kRowWords;
  int b1, b2;
  joint_bodies(d, D, ord, b1, b2);
  // J zero, c = 0, cfm = the world's, lo / hi unbounded, findex -1 (the
  // stepper's defaults before getInfo2, quickstep.cpp:716-745), in 16-byte
  // stores; the iMJ words are written by the row setup
  static_assert(kRowC == 24 && kRowFindex == 28 && kRowB1 == 29 && kRowB2 == 30 && kRowJoint == 31,
                "row layout of the 16-byte stores");
  for (int r = 0; r < m; ++r) {
    float4* row4 = reinterpret_cast<float4*>(rows + r * kRowWords);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    row4[0] = z;
    row4[1] = z;
    row4[2] = z;
    row4[6] = make_float4(0.f, D.cfm, -INFINITY, INFINITY);
    reinterpret_cast<int4*>(row4)[7] = make_int4(-1, b1, b2, ord);
  }
  Info2 in;
  in.fps = h1;
  in.erp = erp;
  in.rows = rows;
  in.fbase = r0;
  BodyRef B1, B2;
  load_body_ref(d, D.body_off + b1, B1);
  if (b2 >= 0) load_body_ref(d, D.body_off + b2, B2);
  const BodyRef* pB2 = b2 >= 0 ? &B2 : nullptr;
  if (ord < D.njp) {
    const DevJoint& J = d.joints[D.joint_off + ord];
    const DevLimot lm1 = step_limot1(J, stops, ord);
    const JointInfo1 i1 = persistent_info1(J, lm1, B1, pB2);
    LimotForce t1 = limot_force_none(), t2 = limot_force_none();
    persistent_info2(J, lm1, i1, B1, pB2, in, t1, t2);
    // a powered motor pushing against a limit adds force / torque inside
    // getInfo2 (joint.cpp:612-660); concurrent additions are rare and use atomics
    for (int t = 0; t < 2; ++t) {
      const LimotForce& tq = t ? t2 : t1;
      if (!tq.active) continue;
      float* fa = reinterpret_cast<float*>(&d.facc[D.body_off + b1]);
      float* ta = reinterpret_cast<float*>(&d.tacc[D.body_off + b1]);
      for (int k = 0; k < 3; ++k) {
        if (tq.f1[k] != 0.f) atomicAdd(fa + k, tq.f1[k]);
        atomicAdd(ta + k, tq.t1[k]);
      }
      if (b2 >= 0) {
        float* fb = reinterpret_cast<float*>(&d.facc[D.body_off + b2]);
        float* tb = reinterpret_cast<float*>(&d.tacc[D.body_off + b2]);
        for (int k = 0; k < 3; ++k) {
          if (tq.f1[k] != 0.f) atomicAdd(fb + k, -tq.f1[k]);
          atomicAdd(tb + k, tq.t2[k]);
        }
      }
    }
  } else {
    const DevContact& ct = d.contacts[D.contact_off + ord - D.njp];
    contact_info2(ct, d.surfaces[ct.surface], m, B1, pB2, D.min_depth, D.max_vel, in);
  }
  if (dbg_rows)
    for (int r = 0; r < m; ++r) dbg_rows[(size_t)(D.row_off + r0 + r) * kRowWords + kDbgErp] = in.erp;
}

// Phase 4: getInfo1 / getInfo2 over the joints in island order. Returns the
// total row count M (or -1 when it exceeds the world's capacity).
OG_D int phase_rows(const BatchDev& d, const WorldDesc& D, int w, int nj, int nisl, int lane, int step,
                      float* dbg_rows) {
  const float* stops = step_stops(d, D, step);
  const int jl_off = D.joint_off + D.contact_off;
  // pass 1: m per joint, prefix -> first row
  int carry = 0;
  for (int base = 0; base < nj; base += 32) {
    const int k = base + lane;
    int m = 0;
    if (k < nj) {
      const int ord = d.jlist[jl_off + k] & 0x3fffffff;
      if (ord < D.njp) {
        const DevJoint& J = d.joints[D.joint_off + ord];
        const DevLimot lm1 = step_limot1(J, stops, ord);
        BodyRef B1, B2;
        load_body_ref(d, D.body_off + J.b1, B1);
        if (J.b2 >= 0) load_body_ref(d, D.body_off + J.b2, B2);
        m = persistent_info1(J, lm1, B1, J.b2 >= 0 ? &B2 : nullptr).m;
      } else {
        m = contact_info1(d.surfaces[d.contacts[D.contact_off + ord - D.njp].surface]);
      }
      d.jm[jl_off + k] = m;
    }
    const int incl = warp_incl_scan(m, lane);
    if (k < nj) d.jrow[jl_off + k] = carry + incl - m;
    carry += __shfl_sync(kFull, incl, 31);
  }
  const int M = carry;
  if (M > D.row_cap || M > kMaxR) {
    if (lane == 0) atomicOr(&d.status[w], ST_ROW_OVERFLOW);
    return -1;
  }
  __syncwarp();
  for (int i = lane; i <= nisl; i += 32) {
    const int js = d.island_jstart[D.body_off + w + i];
    d.island_rstart[D.body_off + w + i] = (js < nj) ? d.jrow[jl_off + js] : M;
  }
  // pass 2: getInfo2. The effective info->erp of a joint is the erp of the
  // last ball or fixed joint before it in the same island (ball.cpp:59 and
  // fixed.cpp:80 write it into the Info2 block the stepper reuses), else the
  // world erp.
  float erp_carry = D.erp;
  for (int base = 0; base < nj; base += 32) {
    const int k = base + lane;
    int ord = -1;
    bool start = false, is_ball = false;
    float my_erp = 0.f;
    if (k < nj) {
      const int v = d.jlist[jl_off + k];
      ord = v & 0x3fffffff;
      start = (v >> 30) & 1;
      if (ord < D.njp) {
        const DevJoint& J = d.joints[D.joint_off + ord];
        if (J.type == J_BALL || J.type == J_FIXED) { is_ball = true; my_erp = J.erp; }
      }
    }
    const unsigned balls = __ballot_sync(kFull, is_ball);
    const unsigned starts = __ballot_sync(kFull, start);
    const unsigned le = (lane == 31) ? kFull : ((1u << (lane + 1)) - 1u);
    const unsigned lt = (1u << lane) - 1u;
    // erp seen by this joint: ball / fixed joints strictly before it within its island
    const unsigned b_lt = balls & lt;
    const unsigned s_le = starts & le;
    const int last_ball = b_lt ? 31 - __clz(b_lt) : -1;
    const int last_start = s_le ? 31 - __clz(s_le) : -1;
    const float ball_erp = __shfl_sync(kFull, my_erp, last_ball < 0 ? 0 : last_ball);
    float erp;
    if (last_ball >= 0 && last_ball >= last_start) erp = ball_erp;
    else if (last_start >= 0) erp = D.erp;
    else erp = erp_carry;
    // carry for the next chunk: the erp after lane 31's joint
    {
      const unsigned b_all = balls, s_all = starts;
      const int lb = b_all ? 31 - __clz(b_all) : -1;
      const int ls = s_all ? 31 - __clz(s_all) : -1;
      const float lb_erp = __shfl_sync(kFull, my_erp, lb < 0 ? 0 : lb);
      if (lb >= 0 && lb >= ls) erp_carry = lb_erp;
      else if (ls >= 0) erp_carry = D.erp;
    }
    if (k < nj)
      assemble_joint_rows(d, D, ord, d.jrow[jl_off + k], d.jm[jl_off + k], erp, stops, dbg_rows);
  }
  __syncwarp();
  return M;
}

// Phase 5 (quickstep.cpp:836-857): tmp1 = invM * fe + v / h of one body
// (global index gb), written to out[6].
OG_D void body_tmp1(const BatchDev& d, int gb, float h1, float* out) {
  const float4 f = d.facc[gb], t = d.tacc[gb], lv = d.lvel[gb], av = d.avel[gb];
  const float im = d.invMass[gb];
  float* t1 = out;
  t1[0] = f.x * im + lv.x * h1;
  t1[1] = f.y * im + lv.y * h1;
  t1[2] = f.z * im + lv.z * h1;
  const float* iw = d.invIw + 12 * gb;
  const float t3[3] = {t.x, t.y, t.z};
  float r3[3];
  mul0_331(r3, iw, t3);
  t1[3] = r3[0] + av.x * h1;
  t1[4] = r3[1] + av.y * h1;
  t1[5] = r3[2] + av.z * h1;
}

// Phase 5 for one row (world-local index r): rhs = c / h - J tmp1, cfm / h,
// iMJ = invM J^T, Ad = w / (J iMJ + cfm), then J, rhs and cfm scaled by Ad
// (quickstep.cpp:117-136, :370-402). tmp1 holds 6 floats per world-local body.
OG_D void row_setup(const BatchDev& d, const WorldDesc& D, int r, const float* tmp1, float h1, float sor_w,
                    float* dbg_rows, float* jcopy) {
  float* row = d.rows + (size_t)(D.row_off + r) * kRowWords;
  float4* row4 = reinterpret_cast<float4*>(row);
  float J[12];
  {
    const float4 a = row4[0], b = row4[1], c = row4[2];
    J[0] = a.x; J[1] = a.y; J[2] = a.z; J[3] = a.w;
    J[4] = b.x; J[5] = b.y; J[6] = b.z; J[7] = b.w;
    J[8] = c.x; J[9] = c.y; J[10] = c.z; J[11] = c.w;
  }
  const float4 w6 = row4[6];
  const int4 w7 = reinterpret_cast<const int4*>(row4)[7];
  const int b1 = w7.y, b2 = w7.z;
  // multiply_J: rhs = J * tmp1
  float sum = 0.f;
  {
    const float* in = tmp1 + 6 * b1;
    for (int j = 0; j < 6; ++j) sum += J[j] * in[j];
    if (b2 != -1) {
      in = tmp1 + 6 * b2;
      for (int j = 0; j < 6; ++j) sum += J[6 + j] * in[j];
    }
  }
  const float rhs = w6.x * h1 - sum;
  const float cfm = w6.y * h1;
  if (jcopy) {
    float4* o = reinterpret_cast<float4*>(jcopy + (size_t)(D.row_off + r) * 12);
    o[0] = make_float4(J[0], J[1], J[2], J[3]);
    o[1] = make_float4(J[4], J[5], J[6], J[7]);
    o[2] = make_float4(J[8], J[9], J[10], J[11]);
  }
  if (dbg_rows) {
    float* o = dbg_rows + (size_t)(D.row_off + r) * kRowWords;
    for (int q = 0; q < 12; ++q) o[q] = J[q];
    o[kRowC] = rhs; o[kRowCfm] = cfm; o[kRowLo] = w6.z; o[kRowHi] = w6.w;
    reinterpret_cast<int*>(o)[kRowFindex] = w7.x;
    reinterpret_cast<int*>(o)[kRowB1] = b1;
    reinterpret_cast<int*>(o)[kRowB2] = b2;
    reinterpret_cast<int*>(o)[kRowJoint] = w7.w;
  }
  // compute_invM_JT
  float iMJ[12];
  {
    const int g1 = D.body_off + b1;
    const float k1 = d.invMass[g1];
    for (int j = 0; j < 3; ++j) iMJ[j] = k1 * J[j];
    mul0_331(iMJ + 3, d.invIw + 12 * g1, J + 3);
    if (b2 != -1) {
      const int g2 = D.body_off + b2;
      const float k2 = d.invMass[g2];
      for (int j = 0; j < 3; ++j) iMJ[6 + j] = k2 * J[6 + j];
      mul0_331(iMJ + 9, d.invIw + 12 * g2, J + 9);
    } else {
      for (int j = 6; j < 12; ++j) iMJ[j] = 0.f;
    }
  }
  float s = 0.f;
  for (int j = 0; j < 6; ++j) s += iMJ[j] * J[j];
  if (b2 != -1)
    for (int j = 6; j < 12; ++j) s += iMJ[j] * J[j];
  const float Ad = sor_w / (s + cfm);
  if (dbg_rows) dbg_rows[(size_t)(D.row_off + r) * kRowWords + kDbgAd] = Ad;
  for (int j = 0; j < 12; ++j) J[j] *= Ad;
  row4[0] = make_float4(J[0], J[1], J[2], J[3]);
  row4[1] = make_float4(J[4], J[5], J[6], J[7]);
  row4[2] = make_float4(J[8], J[9], J[10], J[11]);
  row4[3] = make_float4(iMJ[0], iMJ[1], iMJ[2], iMJ[3]);
  row4[4] = make_float4(iMJ[4], iMJ[5], iMJ[6], iMJ[7]);
  row4[5] = make_float4(iMJ[8], iMJ[9], iMJ[10], iMJ[11]);
  row4[6] = make_float4(rhs * Ad, Ad * cfm, w6.z, w6.w);
}

// Phase 5 over a world's rows; tmp1 per body is staged in S.fc first.
OG_D void phase_row_setup(const BatchDev& d, const WorldDesc& D, int M, const WarpSmem& S, int lane,
                          float* dbg_rows, float* jcopy) {
  const float h1 = 1.0f / D.dt;
  for (int b = lane; b < D.nb; b += 32) body_tmp1(d, D.body_off + b, h1, S.fc + 6 * b);
  __syncwarp();
  const float sor_w = D.sor_w;
  for (int r = lane; r < M; r += 32) row_setup(d, D, r, S.fc, h1, sor_w, dbg_rows, jcopy);
  __syncwarp();
}

// Joint feedback (quickstep.cpp:918-957, Multiply1_12q1 :70-101): for every
// persistent joint, f1 t1 = J1^T lambda and f2 t2 = J2^T lambda over its rows,
// with J as getInfo2 produced it; one lane per joint sums its rows in order.
// A joint without a second body gets f2 = t2 = 0.
OG_D void phase_feedback(const BatchDev& d, const WorldDesc& D, int w, const float* lambda, const float* jcopy,
                         float* feedback, float* contact_feedback, int lane) {
  const int jl_off = D.joint_off + D.contact_off;
  const int nisl = d.nislands[w];
  const int nj = d.island_jstart[D.body_off + w + nisl];
  for (int k = lane; k < nj; k += 32) {
    const int ord = d.jlist[jl_off + k] & 0x3fffffff;
    float* o;
    int b2;
    if (ord < D.njp) {
      if (!feedback) continue;
      o = feedback + (size_t)(D.joint_off + ord) * 12;
      b2 = d.joints[D.joint_off + ord].b2;
    } else {
      if (!contact_feedback) continue;
      o = contact_feedback + (size_t)(D.contact_off + ord - D.njp) * 12;
      b2 = d.contacts[D.contact_off + ord - D.njp].b2;
    }
    const int r0 = d.jrow[jl_off + k], m = d.jm[jl_off + k];
    float f[12];
    for (int q = 0; q < 12; ++q) f[q] = 0.f;
    for (int r = r0; r < r0 + m; ++r) {
      const float s = lambda[r];
      const float* J = jcopy + (size_t)(D.row_off + r) * 12;
      for (int q = 0; q < 12; ++q) f[q] += J[q] * s;
    }
    if (b2 < 0)
      for (int q = 6; q < 12; ++q) f[q] = 0.f;
    for (int q = 0; q < 12; ++q) o[q] = f[q];
  }
}

// sinc for the finite rotation (util.cpp:242-248): the two-term Taylor series
// below 1e-4 (compared in double there, as here)
OG_D float step_sinc(float x) {
  return fabs((double)x) < 1.0e-4 ? 1.0f - x * x * 0.166666666666666666667f : sinf(x) / x;
}
// q += hq * dWtoDQ(w, q) (rotation.cpp dWtoDQ)
OG_D void add_wq(float q[4], float wx, float wy, float wz, float hq) {
  float dq[4];
  dq[0] = 0.5f * (-wx * q[1] - wy * q[2] - wz * q[3]);
  dq[1] = 0.5f * (wx * q[0] + wy * q[3] - wz * q[2]);
  dq[2] = 0.5f * (-wx * q[3] + wy * q[0] + wz * q[1]);
  dq[3] = 0.5f * (wx * q[2] - wy * q[1] + wz * q[0]);
  for (int j = 0; j < 4; j++) q[j] += hq * dq[j];
}
// dxStepBody (util.cpp:255-360) after the velocity update: the angular speed
// cap, the position, the rotation (infinitesimal, or finite about w or about
// the body's axis, with the reference's halved h for the remainder about the
// axis), normalisation, then the velocity damping. Writes the body back;
// returns true when the new state is not finite.
OG_D bool step_body(const BatchDev& d, int gb, float h, float4 lv, float4 av) {
  const float4* bs = d.bstep ? d.bstep + (size_t)kStepRec * gb : nullptr;
  const int fl = bs ? __float_as_int(bs[0].x) : 0;
  if (fl & kStepMaxAng) {
    const float mx = bs[0].y;
    const float a2 = av.x * av.x + av.y * av.y + av.z * av.z;
    if (a2 > mx * mx) {
      const float c = mx / sqrtf(a2);
      av.x *= c; av.y *= c; av.z *= c;
    }
  }
  float4 p = d.pos[gb];
  p.x += h * lv.x; p.y += h * lv.y; p.z += h * lv.z;
  const float4 q4 = d.q[gb];
  float q[4] = {q4.x, q4.y, q4.z, q4.w};
  if (fl & kStepFiniteRot) {
    float r[4], irv[3] = {0.f, 0.f, 0.f};
    const float hh = h * 0.5f;
    if (fl & kStepFiniteAxis) {
      const float ax = bs[1].z, ay = bs[1].w, az = bs[2].x;
      const float k = ax * av.x + ay * av.y + az * av.z;
      const float frv[3] = {ax * k, ay * k, az * k};
      irv[0] = av.x - frv[0]; irv[1] = av.y - frv[1]; irv[2] = av.z - frv[2];
      const float theta = k * hh;
      r[0] = cosf(theta);
      const float sn = step_sinc(theta) * hh;
      r[1] = frv[0] * sn; r[2] = frv[1] * sn; r[3] = frv[2] * sn;
    } else {
      const float wlen = sqrtf(av.x * av.x + av.y * av.y + av.z * av.z);
      const float theta = wlen * hh;
      r[0] = cosf(theta);
      const float sn = step_sinc(theta) * hh;
      r[1] = av.x * sn; r[2] = av.y * sn; r[3] = av.z * sn;
    }
    const float q2[4] = {r[0] * q[0] - r[1] * q[1] - r[2] * q[2] - r[3] * q[3],   // dQMultiply0
                         r[0] * q[1] + r[1] * q[0] + r[2] * q[3] - r[3] * q[2],
                         r[0] * q[2] + r[2] * q[0] + r[3] * q[1] - r[1] * q[3],
                         r[0] * q[3] + r[3] * q[0] + r[1] * q[2] - r[2] * q[1]};
    for (int j = 0; j < 4; j++) q[j] = q2[j];
    if (fl & kStepFiniteAxis) add_wq(q, irv[0], irv[1], irv[2], hh);
  } else {
    add_wq(q, av.x, av.y, av.z, h);
  }
  normalize4(q);
  if (fl & kStepLinDamp) {
    if (lv.x * lv.x + lv.y * lv.y + lv.z * lv.z > bs[0].w) {
      const float k = 1.f - bs[0].z;
      lv.x *= k; lv.y *= k; lv.z *= k;
    }
  }
  if (fl & kStepAngDamp) {
    if (av.x * av.x + av.y * av.y + av.z * av.z > bs[1].y) {
      const float k = 1.f - bs[1].x;
      av.x *= k; av.y *= k; av.z *= k;
    }
  }
  d.pos[gb] = p;
  d.q[gb] = make_float4(q[0], q[1], q[2], q[3]);
  d.lvel[gb] = lv;
  d.avel[gb] = av;
  return !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(lv.x) && isfinite(lv.y) &&
           isfinite(lv.z) && isfinite(av.x) && isfinite(av.y) && isfinite(av.z));
}

// Phase 7 for one body (global index gb): velocity update from the
// constraint forces cforce[6] (null: none) and the external forces, then
// dxStepBody (quickstep.cpp:905-916, :960-975, :1001-1021; util.cpp:255-360).
// Returns true when the new state is not finite.
OG_D bool integrate_body(const BatchDev& d, const WorldDesc& D, int gb, const float* cforce) {
  const float h = D.dt;
  float4 lv = d.lvel[gb], av = d.avel[gb];
  if (cforce) {
    const float* fc = cforce;
    lv.x += h * fc[0]; lv.y += h * fc[1]; lv.z += h * fc[2];
    av.x += h * fc[3]; av.y += h * fc[4]; av.z += h * fc[5];
  }
  const float4 f = d.facc[gb];
  float4 t = d.tacc[gb];
  const float hm = h * d.invMass[gb];
  lv.x += hm * f.x; lv.y += hm * f.y; lv.z += hm * f.z;
  t.x *= h; t.y *= h; t.z *= h;
  {
    const float t3[3] = {t.x, t.y, t.z};
    float r3[3];
    mul0_331(r3, d.invIw + 12 * gb, t3);
    av.x = av.x + r3[0]; av.y = av.y + r3[1]; av.z = av.z + r3[2];
  }
  return step_body(d, gb, h, lv, av);
}
OG_D void phase_integrate(const BatchDev& d, const WorldDesc& D, int w, const float* cforce, int lane,
                          bool have_rows) {
  bool bad = false;
  for (int b = lane; b < D.nb; b += 32)
    bad |= integrate_body(d, D, D.body_off + b, have_rows ? cforce + 6 * b : nullptr);
  if (__any_sync(kFull, bad) && lane == 0) atomicOr(&d.status[w], ST_NONFINITE);
}

// Phase 0: per-step controls into the accumulators, in the reference's order
// (the caller's dBodyAdd* / dJointAdd*Torque calls precede dWorldQuickStep).
// the body forces of the step (global body index gb), replacing last step's accumulators
OG_D void controls_body(const BatchDev& d, int step, int gb) {
  const int nbt = d.world[d.n_worlds - 1].body_off + d.world[d.n_worlds - 1].nb;
  const int cs = d.n_ctrl_steps > 0 ? step % d.n_ctrl_steps : 0;
  float4 f = make_float4(0.f, 0.f, 0.f, 0.f), t = make_float4(0.f, 0.f, 0.f, 0.f);
  if (d.body_force && d.n_ctrl_steps > 0) {
    const float* bf = d.body_force + ((size_t)cs * nbt + gb) * 6;
    f = make_float4(bf[0], bf[1], bf[2], 0.f);
    t = make_float4(bf[3], bf[4], bf[5], 0.f);
  }
  d.facc[gb] = f;
  d.tacc[gb] = t;
}

// the joint torques / forces of the step, added joint by joint in creation
// order (one thread)
OG_D void controls_joints(const BatchDev& d, const WorldDesc& D, int step) {
  const int njt = d.world[d.n_worlds - 1].joint_off + d.world[d.n_worlds - 1].njp;
  const int cs = d.n_ctrl_steps > 0 ? step % d.n_ctrl_steps : 0;
  if (d.joint_torque && d.n_ctrl_steps > 0) {
    for (int j = 0; j < D.njp; ++j) {
      const DevJoint& J = d.joints[D.joint_off + j];
      const float* tq = d.joint_torque + ((size_t)cs * njt + D.joint_off + j) * 2;
      if (J.type == J_HINGE) {
        // dJointAddHingeTorque (ode/src/joints/hinge.cpp:326-345)
        float torque = tq[0];
        if (J.reverse) torque = -torque;
        float R[12], ax[3];
        body_R(d, D.body_off + J.b1, R);
        mul0_331(ax, R, J.axis1);
        ax[0] *= torque; ax[1] *= torque; ax[2] *= torque;
        float4 t1 = d.tacc[D.body_off + J.b1];
        t1.x += ax[0]; t1.y += ax[1]; t1.z += ax[2];
        d.tacc[D.body_off + J.b1] = t1;
        if (J.b2 >= 0) {
          float4 t2 = d.tacc[D.body_off + J.b2];
          t2.x += -ax[0]; t2.y += -ax[1]; t2.z += -ax[2];
          d.tacc[D.body_off + J.b2] = t2;
        }
      } else if (J.type == J_HINGE2 && J.b2 >= 0) {
        // dJointAddHinge2Torques (ode/src/joints/hinge2.cpp:393-410)
        float R1[12], R2[12], a1[3], a2[3];
        body_R(d, D.body_off + J.b1, R1);
        body_R(d, D.body_off + J.b2, R2);
        mul0_331(a1, R1, J.axis1);
        mul0_331(a2, R2, J.axis2);
        float t[3];
        t[0] = a1[0] * tq[0] + a2[0] * tq[1];
        t[1] = a1[1] * tq[0] + a2[1] * tq[1];
        t[2] = a1[2] * tq[0] + a2[2] * tq[1];
        float4 t1 = d.tacc[D.body_off + J.b1];
        t1.x += t[0]; t1.y += t[1]; t1.z += t[2];
        d.tacc[D.body_off + J.b1] = t1;
        float4 t2 = d.tacc[D.body_off + J.b2];
        t2.x += -t[0]; t2.y += -t[1]; t2.z += -t[2];
        d.tacc[D.body_off + J.b2] = t2;
      } else if (J.type == J_SLIDER) {
        // dJointAddSliderForce (ode/src/joints/slider.cpp:305-342); on a
        // reversed joint the reference computes force -= force, i.e. zero
        float force = tq[0];
        if (J.reverse) force -= force;
        float R[12], ax[3];
        body_R(d, D.body_off + J.b1, R);
        mul0_331(ax, R, J.axis1);
        ax[0] *= force; ax[1] *= force; ax[2] *= force;
        float4 f1 = d.facc[D.body_off + J.b1];
        f1.x += ax[0]; f1.y += ax[1]; f1.z += ax[2];
        d.facc[D.body_off + J.b1] = f1;
        if (J.b2 >= 0) {
          float4 f2 = d.facc[D.body_off + J.b2];
          f2.x += -ax[0]; f2.y += -ax[1]; f2.z += -ax[2];
          d.facc[D.body_off + J.b2] = f2;
          // linear torque decoupling: both bodies get (x2 - x1)/2 x force
          const float4 p1 = d.pos[D.body_off + J.b1], p2 = d.pos[D.body_off + J.b2];
          const float c[3] = {0.5f * (p2.x - p1.x), 0.5f * (p2.y - p1.y), 0.5f * (p2.z - p1.z)};
          float ltd[3];
          cross3(ltd, c, ax);
          float4 t1 = d.tacc[D.body_off + J.b1];
          t1.x += ltd[0]; t1.y += ltd[1]; t1.z += ltd[2];
          d.tacc[D.body_off + J.b1] = t1;
          float4 t2 = d.tacc[D.body_off + J.b2];
          t2.x += ltd[0]; t2.y += ltd[1]; t2.z += ltd[2];
          d.tacc[D.body_off + J.b2] = t2;
        }
      } else if (J.type == J_AMOTOR && J.am_num > 0) {
        // dJointAddAMotorTorques(j, tq[0], tq[1], 0) (ode/src/joints/amotor.cpp:474-504)
        BodyRef A1, A2;
        load_body_ref(d, D.body_off + J.b1, A1);
        if (J.b2 >= 0) load_body_ref(d, D.body_off + J.b2, A2);
        float ax[3][3];
        amotor_axes(A1, J.b2 >= 0 ? &A2 : nullptr, J, ax);
        float t[3] = {ax[0][0] * tq[0], ax[0][1] * tq[0], ax[0][2] * tq[0]};
        if (J.am_num >= 2) {
          t[0] += ax[1][0] * tq[1]; t[1] += ax[1][1] * tq[1]; t[2] += ax[1][2] * tq[1];
          if (J.am_num >= 3) { t[0] += ax[2][0] * 0.f; t[1] += ax[2][1] * 0.f; t[2] += ax[2][2] * 0.f; }
        }
        float4 t1 = d.tacc[D.body_off + J.b1];
        t1.x += t[0]; t1.y += t[1]; t1.z += t[2];
        d.tacc[D.body_off + J.b1] = t1;
        if (J.b2 >= 0) {
          float4 t2 = d.tacc[D.body_off + J.b2];
          t2.x += -t[0]; t2.y += -t[1]; t2.z += -t[2];
          d.tacc[D.body_off + J.b2] = t2;
        }
      } else if (J.type == J_UNIVERSAL) {
        // dJointAddUniversalTorques (ode/src/joints/universal.cpp:729-754)
        float tq1 = tq[0], tq2 = tq[1];
        if (J.reverse) { const float tmp = tq1; tq1 = -tq2; tq2 = -tmp; }
        float R1[12], a1[3], a2[3];
        body_R(d, D.body_off + J.b1, R1);
        mul0_331(a1, R1, J.axis1);
        if (J.b2 >= 0) {
          float R2[12];
          body_R(d, D.body_off + J.b2, R2);
          mul0_331(a2, R2, J.axis2);
        } else {
          a2[0] = J.axis2[0]; a2[1] = J.axis2[1]; a2[2] = J.axis2[2];
        }
        float t[3];
        t[0] = a1[0] * tq1 + a2[0] * tq2;
        t[1] = a1[1] * tq1 + a2[1] * tq2;
        t[2] = a1[2] * tq1 + a2[2] * tq2;
        float4 t1 = d.tacc[D.body_off + J.b1];
        t1.x += t[0]; t1.y += t[1]; t1.z += t[2];
        d.tacc[D.body_off + J.b1] = t1;
        if (J.b2 >= 0) {
          float4 t2 = d.tacc[D.body_off + J.b2];
          t2.x += -t[0]; t2.y += -t[1]; t2.z += -t[2];
          d.tacc[D.body_off + J.b2] = t2;
        }
      }
    }
  }
}

OG_D void phase_controls(const BatchDev& d, const WorldDesc& D, int step, int lane) {
  for (int b = lane; b < D.nb; b += 32) controls_body(d, step, D.body_off + b);
  __syncwarp();
  if (lane == 0) controls_joints(d, D, step);
  __syncwarp();
}

struct StepOptions {
  int collide;          // 0: contacts were supplied by the host (ODE API path)
  float* dbg_rows;      // optional: rows before scaling (parity taps)
  float* dbg_lambda;    // optional: lambda after SOR, by world row
  float* dbg_fc;        // optional: cforce per body
  int host_forces;      // 1: facc/tacc were uploaded (skip the control phase)
  int host_adjacency;   // 1: padj holds every joint of each body in list order
  float* jcopy;         // optional: J of every row before scaling, 12 per row (feedback)
  float* feedback;      // optional: [nj_total][12] f1 t1 f2 t2 of the persistent joints
  float* contact_feedback;  // optional: [contact_cap_total][12] the same for contact joints
};

// Setup kernel body: phases 0-5. Leaves the rows, island table, row count
// and island count of the step in global memory for world_solve.
OG_D void world_collide(const BatchDev& d, int w, int step, const WarpSmem& S, int lane,
                        const StepOptions& opt) {
  const WorldDesc D = d.world[w];
  if (!opt.host_forces) phase_controls(d, D, step, lane);
  if (opt.collide) {
    const int nc = phase_collide(d, D, w, S, lane);
    if (lane == 0) d.ncontacts[w] = nc;
  }
  __syncwarp();
  phase_body_prologue(d, D, lane);
  __syncwarp();
}

OG_D void world_setup(const BatchDev& d, int w, int step, const WarpSmem& S, int lane, const StepOptions& opt) {
  const WorldDesc D = d.world[w];
  const int nc = d.ncontacts[w];
  int M = 0, nisl = 0;
  if (D.njp + nc > kMaxR) {
    if (lane == 0) atomicOr(&d.status[w], ST_TOO_LARGE);
    M = -1;
  } else {
    const int nj = phase_islands(d, D, w, opt.host_adjacency ? 0 : nc, D.njp + nc, S, lane, &nisl);
    M = phase_rows(d, D, w, nj, nisl, lane, step, opt.dbg_rows);
  }
  if (M > 0) phase_row_setup(d, D, M, S, lane, opt.dbg_rows, opt.jcopy);
  if (lane == 0) {
    d.nrows[w] = M < 0 ? 0 : M;
    d.nislands[w] = M > 0 ? nisl : 0;
  }
  __syncwarp();
}

// Solve kernel body: phase 6 (SOR) and phase 7 (integration). smem: the
// warp's kFwdSmemPerWarp bytes of shared memory.
OG_D void world_solve(const BatchDev& d, int w, unsigned char* smem, int lane, const StepOptions& opt) {
  const WorldDesc D = d.world[w];
  const int M = d.nrows[w];
  const int nisl = d.nislands[w];
  unsigned seed = d.seed[w];
  unsigned char* scratch =
      D.fwd_scratch >= 0 ? d.fwd_scratch + (size_t)D.fwd_scratch * kFwdScratchPerWorld : nullptr;
  const FwdSmem S = carve_fwd(smem, M, scratch);
  const bool have_rows = M > 0 && M <= S.cap;
  if (M > S.cap) {
    if (lane == 0) atomicOr(&d.status[w], ST_ROW_OVERFLOW);
    for (int i = lane; i < (kMaxB + 1) * 6; i += 32) S.fc[i] = 0.f;
    __syncwarp();
  }
  if (have_rows) {
    const float* rows = d.rows + (size_t)D.row_off * kRowWords;
    const int* rstart = d.island_rstart + D.body_off + w;
    float4* sweep = d.sweep + (size_t)(D.row_off + 32 * w) * 8;
    seed = fwd_sor_world(rows, rstart, D.nb, M, nisl, D.iterations, seed, S, lane, sweep, D.row_cap + 32);
    __syncwarp();
    if (opt.dbg_lambda)
      for (int r = lane; r < M; r += 32) opt.dbg_lambda[D.row_off + r] = S.lambda[r];
    if (opt.dbg_fc)
      for (int i = lane; i < D.nb * 6; i += 32) opt.dbg_fc[(size_t)D.body_off * 6 + i] = S.fc[i];
    if ((opt.feedback || opt.contact_feedback) && opt.jcopy)
      phase_feedback(d, D, w, S.lambda, opt.jcopy, opt.feedback, opt.contact_feedback, lane);
  }
  if (lane == 0) d.seed[w] = seed;
  phase_integrate(d, D, w, S.fc, lane, have_rows);
  __syncwarp();
}

}  // namespace og
