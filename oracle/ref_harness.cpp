/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE. Drives the unmodified reference
 * ODE 0.12 (built from its own sources by oracle/Makefile into oracle/_ref/)
 * through its PUBLIC C API only, on a scene described by odegpuScene, and
 * records what the public API can observe. Nothing in the product links this.
 *
 * Per world and step it performs exactly the canonical sequence documented in
 * include/odegpu_scene.h:
 *   1. dCollide over geom pairs (i<j) in index order  (collision_kernel.cpp:292),
 *      skipping bodies joined by a non-contact joint (dAreConnectedExcluding,
 *      ode.cpp:1529, as ODE's demos do in their near-callbacks)
 *   2. dJointCreateContact + dJointAttach(body(gi), body(gj)) per contact
 *      (ode.cpp:1201, :1348)
 *   3. per-step controls via dJointAdd{Hinge,Hinge2,Universal}Torque(s) /
 *      dJointAddSliderForce /
 *      dBodyAddForce / dBodyAddTorque
 *   4. dWorldQuickStep (ode.cpp:1807)
 *   5. dJointGroupEmpty (ode.cpp:1305)
 */
#include <ode/ode.h>
#include <cmath>
#include <string.h>
#include <stdlib.h>
#include "odegpu_scene.h"

extern "C" {

/* Output record per contact: pos[3], normal[3], depth, gi, gj (as doubles). */
#define REF_CONTACT_REC 9
/* Output record per body and step: pos[3], q[4], lvel[3], avel[3]. */
#define REF_BODY_REC 13

static void read_body(dBodyID b, double* out) {
  const dReal* p = dBodyGetPosition(b);
  const dReal* q = dBodyGetQuaternion(b);
  const dReal* v = dBodyGetLinearVel(b);
  const dReal* w = dBodyGetAngularVel(b);
  for (int k = 0; k < 3; ++k) out[k] = p[k];
  for (int k = 0; k < 4; ++k) out[3 + k] = q[k];
  for (int k = 0; k < 3; ++k) out[7 + k] = v[k];
  for (int k = 0; k < 3; ++k) out[10 + k] = w[k];
}

static void set_limot(dJointID j, int group, const double* p,
                      void (*setp)(dJointID, int, dReal)) {
  /* ODE's dJointSet*Param with parameter numbers relative to a group
   * (include/ode/common.h:305-354). Order matters only through dParamFMax's
   * "value >= 0" guard, which we respect by passing real values. */
  const int base = group * 0x100;
  setp(j, base + dParamLoStop, p[0]);
  setp(j, base + dParamHiStop, p[1]);
  setp(j, base + dParamVel, p[2]);
  setp(j, base + dParamFMax, p[3]);
  setp(j, base + dParamFudgeFactor, p[4]);
  setp(j, base + dParamBounce, p[5]);
  setp(j, base + dParamCFM, p[6]);
  setp(j, base + dParamStopERP, p[7]);
  setp(j, base + dParamStopCFM, p[8]);
}

/*
 * Run world `w` of `scene` for n_steps. Outputs (any may be NULL):
 *   state      [(n_steps+1)][nb_w][13]   state after each step (row 0 = initial)
 *   ncontacts  [n_steps]                 contacts created before each step
 *   contacts   [n_steps][max_rec][9]     contact records (first max_rec kept)
 *   feedback   [n_steps][nj_w][12]       dJointFeedback f1,t1,f2,t2 of the
 *                                        persistent joints after each step
 *   seed_out   [n_steps]                 dRandGetSeed after each step
 * Returns 0 on success, -1 on bad arguments.
 */
static int g_exact = 0;   /* 1: dWorldStep (ode.cpp:1787) instead of dWorldQuickStep */
void ref_set_stepper(int exact) { g_exact = exact; }

int ref_run_world(const odegpuScene* sc, int w, int n_steps, double* state,
                  int* ncontacts, double* contacts, int max_rec,
                  double* feedback, unsigned int* seed_out) {
  if (!sc || w < 0 || w >= sc->n_worlds || n_steps < 0) return -1;
  const odegpuWorldParams* P = &sc->world[w];
  const int b0 = sc->body_off[w], nb = sc->body_off[w + 1] - b0;
  const int g0 = sc->geom_off[w], ng = sc->geom_off[w + 1] - g0;
  const int j0 = sc->joint_off[w], nj = sc->joint_off[w + 1] - j0;

  dInitODE2(0);
  dWorldID world = dWorldCreate();
  dWorldSetGravity(world, P->gravity[0], P->gravity[1], P->gravity[2]);
  dWorldSetERP(world, P->erp);
  dWorldSetCFM(world, P->cfm);
  dWorldSetQuickStepNumIterations(world, P->iterations);
  dWorldSetQuickStepW(world, P->sor_w);
  dWorldSetContactMaxCorrectingVel(world, P->max_vel);
  dWorldSetContactSurfaceLayer(world, P->min_depth);

  dBodyID* bodies = (dBodyID*)calloc(nb > 0 ? nb : 1, sizeof(dBodyID));
  for (int i = 0; i < nb; ++i) {
    const int g = b0 + i;
    dBodyID b = dBodyCreate(world);
    bodies[i] = b;
    dBodySetPosition(b, sc->body_pos[3 * g], sc->body_pos[3 * g + 1], sc->body_pos[3 * g + 2]);
    dQuaternion q = {sc->body_q[4 * g], sc->body_q[4 * g + 1], sc->body_q[4 * g + 2],
                     sc->body_q[4 * g + 3]};
    dBodySetQuaternion(b, q);
    dBodySetLinearVel(b, sc->body_lvel[3 * g], sc->body_lvel[3 * g + 1], sc->body_lvel[3 * g + 2]);
    dBodySetAngularVel(b, sc->body_avel[3 * g], sc->body_avel[3 * g + 1], sc->body_avel[3 * g + 2]);
    const double* I = sc->body_I + 9 * g;
    dMass m;
    dMassSetParameters(&m, sc->body_mass[g], 0, 0, 0, I[0], I[4], I[8], I[1], I[2], I[5]);
    dBodySetMass(b, &m);
    const int fl = sc->body_flags[g];
    dBodySetGyroscopicMode(b, (fl & ODEGPU_BODY_GYROSCOPIC) ? 1 : 0);
    dBodySetGravityMode(b, (fl & ODEGPU_BODY_NO_GRAVITY) ? 0 : 1);
  }

  dGeomID* geoms = (dGeomID*)calloc(ng > 0 ? ng : 1, sizeof(dGeomID));
  dHeightfieldDataID* hfd = (dHeightfieldDataID*)calloc(ng > 0 ? ng : 1, sizeof(dHeightfieldDataID));
  for (int i = 0; i < ng; ++i) {
    const int g = g0 + i;
    const double* gp = sc->geom_param + ODEGPU_GEOM_NPARAM * g;
    dGeomID geom = 0;
    switch (sc->geom_type[g]) {
      case ODEGPU_GEOM_SPHERE: geom = dCreateSphere(0, gp[0]); break;
      case ODEGPU_GEOM_BOX: geom = dCreateBox(0, gp[0], gp[1], gp[2]); break;
      case ODEGPU_GEOM_CAPSULE: geom = dCreateCapsule(0, gp[0], gp[1]); break;
      case ODEGPU_GEOM_CYLINDER: geom = dCreateCylinder(0, gp[0], gp[1]); break;
      case ODEGPU_GEOM_PLANE: geom = dCreatePlane(0, gp[0], gp[1], gp[2], gp[3]); break;
      case ODEGPU_GEOM_HEIGHTFIELD: {
        const odegpuHeightfield* H = &sc->heightfields[(int)gp[0]];
        hfd[i] = dGeomHeightfieldDataCreate();
        dGeomHeightfieldDataBuildDouble(hfd[i], H->heights, 1, H->width, H->depth, H->nx,
                                        H->nz, H->scale, H->offset, H->thickness, H->wrap);
        geom = dCreateHeightfield(0, hfd[i], 1);
        dGeomSetPosition(geom, H->pos[0], H->pos[1], H->pos[2]);
        dMatrix3 R = {H->R[0], H->R[1], H->R[2], 0, H->R[3], H->R[4], H->R[5], 0,
                      H->R[6], H->R[7], H->R[8], 0};
        dGeomSetRotation(geom, R);
        break;
      }
      default: free(bodies); free(geoms); free(hfd); dWorldDestroy(world); return -1;
    }
    geoms[i] = geom;
    const int gb = sc->geom_body[g];
    if (gb >= 0) dGeomSetBody(geom, bodies[gb]);
  }

  dJointID* joints = (dJointID*)calloc(nj > 0 ? nj : 1, sizeof(dJointID));
  dJointFeedback* fbs = (dJointFeedback*)calloc(nj > 0 ? nj : 1, sizeof(dJointFeedback));
  for (int i = 0; i < nj; ++i) {
    const int g = j0 + i;
    const int jb1 = sc->joint_body[2 * g], jb2 = sc->joint_body[2 * g + 1];
    dBodyID B1 = jb1 >= 0 ? bodies[jb1] : 0, B2 = jb2 >= 0 ? bodies[jb2] : 0;
    const double* a = sc->joint_anchor + 3 * g;
    const double* x1 = sc->joint_axis1 + 3 * g;
    const double* x2 = sc->joint_axis2 + 3 * g;
    const double* jp = sc->joint_param + ODEGPU_JOINT_NPARAM * g;
    dJointID j = 0;
    switch (sc->joint_type[g]) {
      case ODEGPU_JOINT_BALL:
        j = dJointCreateBall(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetBallAnchor(j, a[0], a[1], a[2]);
        dJointSetBallParam(j, dParamERP, jp[0]);
        dJointSetBallParam(j, dParamCFM, jp[1]);
        break;
      case ODEGPU_JOINT_HINGE:
        j = dJointCreateHinge(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetHingeAnchor(j, a[0], a[1], a[2]);
        dJointSetHingeAxis(j, x1[0], x1[1], x1[2]);
        set_limot(j, 0, jp, dJointSetHingeParam);
        break;
      case ODEGPU_JOINT_HINGE2:
        j = dJointCreateHinge2(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetHinge2Anchor(j, a[0], a[1], a[2]);
        dJointSetHinge2Axis1(j, x1[0], x1[1], x1[2]);
        dJointSetHinge2Axis2(j, x2[0], x2[1], x2[2]);
        set_limot(j, 0, jp, dJointSetHinge2Param);
        set_limot(j, 1, jp + 9, dJointSetHinge2Param);
        dJointSetHinge2Param(j, dParamSuspensionERP, jp[18]);
        dJointSetHinge2Param(j, dParamSuspensionCFM, jp[19]);
        break;
      case ODEGPU_JOINT_SLIDER:
        j = dJointCreateSlider(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetSliderAxis(j, x1[0], x1[1], x1[2]);
        set_limot(j, 0, jp, dJointSetSliderParam);
        break;
      case ODEGPU_JOINT_UNIVERSAL:
        j = dJointCreateUniversal(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetUniversalAnchor(j, a[0], a[1], a[2]);
        dJointSetUniversalAxis1(j, x1[0], x1[1], x1[2]);
        dJointSetUniversalAxis2(j, x2[0], x2[1], x2[2]);
        set_limot(j, 0, jp, dJointSetUniversalParam);
        set_limot(j, 1, jp + 9, dJointSetUniversalParam);
        break;
      case ODEGPU_JOINT_AMOTOR: {
        j = dJointCreateAMotor(world, 0);
        dJointAttach(j, B1, B2);
        const int mode = (int)jp[1];
        dJointSetAMotorMode(j, mode);
        dJointSetAMotorNumAxes(j, (int)jp[0]);
        const double* ax[3] = {a, x1, x2};
        const int num = dJointGetAMotorNumAxes(j);
        for (int k = 0; k < 3; ++k)
          if (mode == dAMotorEuler ? k != 1 : k < num)
            dJointSetAMotorAxis(j, k, (int)jp[2 + k], ax[k][0], ax[k][1], ax[k][2]);
        set_limot(j, 0, jp + 5, dJointSetAMotorParam);
        set_limot(j, 1, jp + 14, dJointSetAMotorParam);
        set_limot(j, 2, jp + 23, dJointSetAMotorParam);
        if (mode == dAMotorUser)
          for (int k = 0; k < num; ++k) dJointSetAMotorAngle(j, k, jp[32 + k]);
        break;
      }
      case ODEGPU_JOINT_FIXED:
        j = dJointCreateFixed(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetFixed(j);
        dJointSetFixedParam(j, dParamERP, jp[0]);
        dJointSetFixedParam(j, dParamCFM, jp[1]);
        break;
      default: break;
    }
    joints[i] = j;
    if (j && feedback) dJointSetFeedback(j, &fbs[i]);
  }

  dJointGroupID group = dJointGroupCreate(0);
  dContactGeom* cg = (dContactGeom*)calloc(16, sizeof(dContactGeom));
  const int maxc = P->max_contacts;
  dRandSetSeed(P->seed);

  if (state) for (int i = 0; i < nb; ++i) read_body(bodies[i], state + REF_BODY_REC * i);

  for (int s = 0; s < n_steps; ++s) {
    int nc = 0;
    for (int i = 0; i < ng; ++i) {
      for (int k = i + 1; k < ng; ++k) {
        const int bi = sc->geom_body[g0 + i], bk = sc->geom_body[g0 + k];
        if (bi < 0 && bk < 0) continue;
        if (bi == bk) continue;
        if (bi >= 0 && bk >= 0 &&
            dAreConnectedExcluding(bodies[bi], bodies[bk], dJointTypeContact))
          continue;
        const int n = dCollide(geoms[i], geoms[k], maxc, cg, sizeof(dContactGeom));
        const int si = sc->geom_surface[g0 + i], sk = sc->geom_surface[g0 + k];
        const odegpuSurface* S = &sc->surfaces[si > sk ? si : sk];
        for (int c = 0; c < n; ++c) {
          dContact con;
          memset(&con, 0, sizeof(con));
          con.surface.mode = S->mode;
          con.surface.mu = S->mu;
          con.surface.mu2 = S->mu2;
          con.surface.bounce = S->bounce;
          con.surface.bounce_vel = S->bounce_vel;
          con.surface.soft_erp = S->soft_erp;
          con.surface.soft_cfm = S->soft_cfm;
          con.surface.motion1 = S->motion1;
          con.surface.motion2 = S->motion2;
          con.surface.motionN = S->motionN;
          con.surface.slip1 = S->slip1;
          con.surface.slip2 = S->slip2;
          con.geom = cg[c];
          dJointID cj = dJointCreateContact(world, group, &con);
          dJointAttach(cj, bi >= 0 ? bodies[bi] : 0, bk >= 0 ? bodies[bk] : 0);
          if (contacts && nc < max_rec) {
            double* r = contacts + ((size_t)s * max_rec + nc) * REF_CONTACT_REC;
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
    if (ncontacts) ncontacts[s] = nc;

    if (sc->n_ctrl_steps > 0) {
      const int cs = s % sc->n_ctrl_steps;
      if (sc->joint_stop) {
        for (int i = 0; i < nj; ++i) {
          const int t = sc->joint_type[j0 + i];
          void (*setp)(dJointID, int, dReal) = 0;
          if (t == ODEGPU_JOINT_HINGE) setp = dJointSetHingeParam;
          else if (t == ODEGPU_JOINT_HINGE2) setp = dJointSetHinge2Param;
          else if (t == ODEGPU_JOINT_SLIDER) setp = dJointSetSliderParam;
          else if (t == ODEGPU_JOINT_UNIVERSAL) setp = dJointSetUniversalParam;
          else if (t == ODEGPU_JOINT_AMOTOR) setp = dJointSetAMotorParam;
          if (!setp) continue;
          const double v = sc->joint_stop[(size_t)cs * sc->joint_off[sc->n_worlds] + j0 + i];
          const double* jp = sc->joint_param + (size_t)(j0 + i) * ODEGPU_JOINT_NPARAM;
          const double* lp = t == ODEGPU_JOINT_AMOTOR ? jp + 5 : jp;
          const double lo = std::isnan(v) ? lp[0] : v, hi = std::isnan(v) ? lp[1] : v;
          setp(joints[i], dParamLoStop, lo);
          setp(joints[i], dParamHiStop, hi);
        }
      }
      if (sc->joint_torque) {
        for (int i = 0; i < nj; ++i) {
          const double* t = sc->joint_torque + ((size_t)cs * sc->joint_off[sc->n_worlds] + j0 + i) * 2;
          const int jt = sc->joint_type[j0 + i];
          if (jt == ODEGPU_JOINT_HINGE) dJointAddHingeTorque(joints[i], t[0]);
          else if (jt == ODEGPU_JOINT_HINGE2) dJointAddHinge2Torques(joints[i], t[0], t[1]);
          else if (jt == ODEGPU_JOINT_SLIDER) dJointAddSliderForce(joints[i], t[0]);
          else if (jt == ODEGPU_JOINT_UNIVERSAL) dJointAddUniversalTorques(joints[i], t[0], t[1]);
          else if (jt == ODEGPU_JOINT_AMOTOR) dJointAddAMotorTorques(joints[i], t[0], t[1], 0);
        }
      }
      if (sc->body_force) {
        for (int i = 0; i < nb; ++i) {
          const double* f = sc->body_force + ((size_t)cs * sc->body_off[sc->n_worlds] + b0 + i) * 6;
          dBodyAddForce(bodies[i], f[0], f[1], f[2]);
          dBodyAddTorque(bodies[i], f[3], f[4], f[5]);
        }
      }
    }

    if (g_exact) dWorldStep(world, P->dt);
    else dWorldQuickStep(world, P->dt);
    dJointGroupEmpty(group);

    if (state)
      for (int i = 0; i < nb; ++i)
        read_body(bodies[i], state + REF_BODY_REC * ((size_t)(s + 1) * nb + i));
    if (feedback) {
      for (int i = 0; i < nj; ++i) {
        double* r = feedback + ((size_t)s * nj + i) * 12;
        for (int q = 0; q < 3; ++q) {
          r[q] = fbs[i].f1[q];
          r[3 + q] = fbs[i].t1[q];
          r[6 + q] = fbs[i].f2[q];
          r[9 + q] = fbs[i].t2[q];
        }
      }
    }
    if (seed_out) seed_out[s] = (unsigned int)dRandGetSeed();
  }

  dJointGroupDestroy(group);
  for (int i = 0; i < nj; ++i)
    if (joints[i]) dJointDestroy(joints[i]);
  for (int i = 0; i < ng; ++i) dGeomDestroy(geoms[i]);
  for (int i = 0; i < ng; ++i)
    if (hfd[i]) dGeomHeightfieldDataDestroy(hfd[i]);
  dWorldDestroy(world);
  dCloseODE();
  free(cg); free(joints); free(fbs); free(geoms); free(hfd); free(bodies);
  return 0;
}

/* dTestRand known-answer test of the reference RNG (ode/src/misc.cpp:52-62),
 * plus raw access to the reference dRand/dRandInt for RNG parity tests. */
int ref_test_rand(void) { return dTestRand(); }
void ref_rand_set_seed(unsigned int s) { dRandSetSeed(s); }
unsigned int ref_rand_get_seed(void) { return (unsigned int)dRandGetSeed(); }
int ref_rand_int(int n) { return dRandInt(n); }

/* Single dCollide call on two standalone geoms with explicit placement, for
 * collider known-answer tests. type/param as in odegpuScene; pos[3], R[9]
 * row-major. Writes up to maxc records of 9 doubles (pos, normal, depth, 0, 0). */
static dGeomID make_geom(int type, const double* p) {
  switch (type) {
    case ODEGPU_GEOM_SPHERE: return dCreateSphere(0, p[0]);
    case ODEGPU_GEOM_BOX: return dCreateBox(0, p[0], p[1], p[2]);
    case ODEGPU_GEOM_CAPSULE: return dCreateCapsule(0, p[0], p[1]);
    case ODEGPU_GEOM_PLANE: return dCreatePlane(0, p[0], p[1], p[2], p[3]);
    case ODEGPU_GEOM_RAY: return dCreateRay(0, p[0]);
    case ODEGPU_GEOM_CYLINDER: return dCreateCylinder(0, p[0], p[1]);
    default: return 0;
  }
}

int ref_collide(int t1, const double* p1, const double* pos1, const double* R1, int t2,
                const double* p2, const double* pos2, const double* R2, int flags,
                double* out) {
  dInitODE2(0);
  dGeomID a = make_geom(t1, p1), b = make_geom(t2, p2);
  if (!a || !b) return -1;
  if (t1 != ODEGPU_GEOM_PLANE) {
    dGeomSetPosition(a, pos1[0], pos1[1], pos1[2]);
    dMatrix3 R = {R1[0], R1[1], R1[2], 0, R1[3], R1[4], R1[5], 0, R1[6], R1[7], R1[8], 0};
    dGeomSetRotation(a, R);
  }
  if (t2 != ODEGPU_GEOM_PLANE) {
    dGeomSetPosition(b, pos2[0], pos2[1], pos2[2]);
    dMatrix3 R = {R2[0], R2[1], R2[2], 0, R2[3], R2[4], R2[5], 0, R2[6], R2[7], R2[8], 0};
    dGeomSetRotation(b, R);
  }
  dContactGeom cg[16];
  const int n = dCollide(a, b, flags, cg, sizeof(dContactGeom));
  for (int c = 0; c < n; ++c) {
    double* r = out + 9 * c;
    for (int q = 0; q < 3; ++q) r[q] = cg[c].pos[q];
    for (int q = 0; q < 3; ++q) r[3 + q] = cg[c].normal[q];
    r[6] = cg[c].depth;
    r[7] = 0;
    r[8] = 0;
  }
  dGeomDestroy(a);
  dGeomDestroy(b);
  dCloseODE();
  return n;
}

/* dCollide(heightfield, geom) with the heightfield placed at H->pos / H->R
 * (placeable), the geom of class t2 at pos2 / R2; same output as ref_collide. */
int ref_collide_hf(const odegpuHeightfield* H, int t2, const double* p2, const double* pos2,
                   const double* R2, int flags, double* out) {
  dInitODE2(0);
  dHeightfieldDataID hd = dGeomHeightfieldDataCreate();
  dGeomHeightfieldDataBuildDouble(hd, H->heights, 1, H->width, H->depth, H->nx, H->nz, H->scale,
                                  H->offset, H->thickness, H->wrap);
  dGeomID a = dCreateHeightfield(0, hd, 1);
  dGeomSetPosition(a, H->pos[0], H->pos[1], H->pos[2]);
  dMatrix3 RH = {H->R[0], H->R[1], H->R[2], 0, H->R[3], H->R[4], H->R[5], 0,
                 H->R[6], H->R[7], H->R[8], 0};
  dGeomSetRotation(a, RH);
  dGeomID b = make_geom(t2, p2);
  if (!b) return -1;
  dGeomSetPosition(b, pos2[0], pos2[1], pos2[2]);
  dMatrix3 R = {R2[0], R2[1], R2[2], 0, R2[3], R2[4], R2[5], 0, R2[6], R2[7], R2[8], 0};
  dGeomSetRotation(b, R);
  dContactGeom cg[64];
  const int n = dCollide(a, b, flags, cg, sizeof(dContactGeom));
  for (int c = 0; c < n; ++c) {
    double* r = out + 9 * c;
    for (int q = 0; q < 3; ++q) r[q] = cg[c].pos[q];
    for (int q = 0; q < 3; ++q) r[3 + q] = cg[c].normal[q];
    r[6] = cg[c].depth;
    r[7] = 0;
    r[8] = 0;
  }
  dGeomDestroy(a);
  dGeomDestroy(b);
  dGeomHeightfieldDataDestroy(hd);
  dCloseODE();
  return n;
}

}  // extern "C"
