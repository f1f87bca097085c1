/*
 * scene_player.c -- a plain ODE program that replays one world of an
 * odegpuScene (bodies, sphere / box / capsule / plane geoms, ball, hinge,
 * slider, universal, hinge2, fixed and angular motor joints, per-step
 * controls) through ODE
 * 0.12's public C API only. Built against the reference (<ode/ode.h>,
 * -DdSINGLE, linked with the reference library) it runs ODE on the CPU; built
 * against include/ode_gpu.h and linked with libodegpu it runs the same calls
 * on the GPU. Per step it follows the canonical sequence of
 * include/odegpu_scene.h: dCollide over geom pairs i < k (skipping static
 * pairs, same-body pairs and jointed bodies), one contact joint per contact
 * with the surface of the higher surface index, the step's joint stops,
 * joint torques / slider forces and body forces, dWorldQuickStep (or dWorldStep),
 * dJointGroupEmpty.
 *
 * Input (text; numbers may be inf / nan):
 *   nb ng nj nsurf nsteps nctrl seed max_contacts
 *   gx gy gz erp cfm iterations sor_w max_vel min_depth dt
 *   nsurf lines:  mode mu mu2 bounce bounce_vel soft_erp soft_cfm motion1 motion2 motionN slip1 slip2
 *   nb lines:     px py pz qw qx qy qz vx vy vz wx wy wz mass I[9] flags
 *   ng lines:     type body surface p0 p1 p2 p3
 *   nj lines:     type b1 b2 anchor[3] axis1[3] axis2[3] param[36]
 *   nctrl blocks: nj lines "torque0 torque1 stop", then nb lines "force[3] torque[3]"
 * Output: one line per body after the last step: pos[3] q[4] lvel[3] avel[3].
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef USE_REFERENCE_ODE
#include <ode/ode.h>
#else
#include "ode_gpu.h"
#endif

enum { SPHERE = 0, BOX = 1, CAPSULE = 2, CYLINDER = 3, PLANE = 4 };
enum { BALL = 1, HINGE = 2, SLIDER = 3, UNIVERSAL = 5, HINGE2 = 6, FIXED = 7, AMOTOR = 9 };
#define NPARAM 36

static int rd(FILE* f, double* v, int n) {
  for (int i = 0; i < n; ++i)
    if (fscanf(f, "%lf", &v[i]) != 1) return 0;
  return 1;
}

typedef void (*setp_fn)(dJointID, int, dReal);

static void set_limot(dJointID j, int group, const double* p, setp_fn setp) {
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

static setp_fn stop_setter(int type) {
  switch (type) {
    case HINGE: return dJointSetHingeParam;
    case HINGE2: return dJointSetHinge2Param;
    case SLIDER: return dJointSetSliderParam;
    case UNIVERSAL: return dJointSetUniversalParam;
    case AMOTOR: return dJointSetAMotorParam;
    default: return 0;
  }
}

int main(int argc, char** argv) {
  FILE* in = argc > 1 ? fopen(argv[1], "r") : stdin;
  /* a second argument "exact" steps with dWorldStep instead of dWorldQuickStep */
  const int exact = argc > 2 && strcmp(argv[2], "exact") == 0;
  double h[8], wp[10];
  if (!in || !rd(in, h, 8) || !rd(in, wp, 10)) return 2;
  const int nb = (int)h[0], ng = (int)h[1], nj = (int)h[2], ns = (int)h[3];
  const int nsteps = (int)h[4], nctrl = (int)h[5], maxc = (int)h[7];
  const unsigned long seed = (unsigned long)h[6];
  if (maxc < 1 || maxc > 16) return 2;

  dInitODE2(0);
  dWorldID world = dWorldCreate();
  dWorldSetGravity(world, wp[0], wp[1], wp[2]);
  dWorldSetERP(world, wp[3]);
  dWorldSetCFM(world, wp[4]);
  dWorldSetQuickStepNumIterations(world, (int)wp[5]);
  dWorldSetQuickStepW(world, wp[6]);
  dWorldSetContactMaxCorrectingVel(world, wp[7]);
  dWorldSetContactSurfaceLayer(world, wp[8]);
  const double dt = wp[9];

  double* surf = (double*)calloc((size_t)(ns > 0 ? ns : 1) * 12, sizeof(double));
  for (int i = 0; i < ns; ++i)
    if (!rd(in, surf + 12 * i, 12)) return 2;

  dBodyID* bodies = (dBodyID*)calloc(nb > 0 ? nb : 1, sizeof(dBodyID));
  for (int i = 0; i < nb; ++i) {
    double b[24];
    if (!rd(in, b, 24)) return 2;
    dBodyID body = dBodyCreate(world);
    bodies[i] = body;
    dBodySetPosition(body, b[0], b[1], b[2]);
    dQuaternion q = {b[3], b[4], b[5], b[6]};
    dBodySetQuaternion(body, q);
    dBodySetLinearVel(body, b[7], b[8], b[9]);
    dBodySetAngularVel(body, b[10], b[11], b[12]);
    const double* I = b + 14;
    dMass m;
    dMassSetParameters(&m, b[13], 0, 0, 0, I[0], I[4], I[8], I[1], I[2], I[5]);
    dBodySetMass(body, &m);
    const int fl = (int)b[23];
    dBodySetGyroscopicMode(body, (fl & 1) ? 1 : 0);
    dBodySetGravityMode(body, (fl & 2) ? 0 : 1);
  }

  dGeomID* geoms = (dGeomID*)calloc(ng > 0 ? ng : 1, sizeof(dGeomID));
  int* gbody = (int*)calloc(ng > 0 ? ng : 1, sizeof(int));
  int* gsurf = (int*)calloc(ng > 0 ? ng : 1, sizeof(int));
  for (int i = 0; i < ng; ++i) {
    double g[7];
    if (!rd(in, g, 7)) return 2;
    const double* p = g + 3;
    dGeomID geom = 0;
    switch ((int)g[0]) {
      case SPHERE: geom = dCreateSphere(0, p[0]); break;
      case BOX: geom = dCreateBox(0, p[0], p[1], p[2]); break;
      case CAPSULE: geom = dCreateCapsule(0, p[0], p[1]); break;
      case CYLINDER: geom = dCreateCylinder(0, p[0], p[1]); break;
      case PLANE: geom = dCreatePlane(0, p[0], p[1], p[2], p[3]); break;
      default: return 2;
    }
    geoms[i] = geom;
    gbody[i] = (int)g[1];
    gsurf[i] = (int)g[2];
    if (gbody[i] >= 0) dGeomSetBody(geom, bodies[gbody[i]]);
  }

  dJointID* joints = (dJointID*)calloc(nj > 0 ? nj : 1, sizeof(dJointID));
  int* jtype = (int*)calloc(nj > 0 ? nj : 1, sizeof(int));
  double* jparam = (double*)calloc((size_t)(nj > 0 ? nj : 1) * NPARAM, sizeof(double));
  for (int i = 0; i < nj; ++i) {
    double r[12];
    if (!rd(in, r, 12) || !rd(in, jparam + NPARAM * i, NPARAM)) return 2;
    const int t = (int)r[0], jb1 = (int)r[1], jb2 = (int)r[2];
    const double *a = r + 3, *x1 = r + 6, *x2 = r + 9, *jp = jparam + NPARAM * i;
    dBodyID B1 = jb1 >= 0 ? bodies[jb1] : 0, B2 = jb2 >= 0 ? bodies[jb2] : 0;
    dJointID j = 0;
    jtype[i] = t;
    switch (t) {
      case BALL:
        j = dJointCreateBall(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetBallAnchor(j, a[0], a[1], a[2]);
        dJointSetBallParam(j, dParamERP, jp[0]);
        dJointSetBallParam(j, dParamCFM, jp[1]);
        break;
      case HINGE:
        j = dJointCreateHinge(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetHingeAnchor(j, a[0], a[1], a[2]);
        dJointSetHingeAxis(j, x1[0], x1[1], x1[2]);
        set_limot(j, 0, jp, dJointSetHingeParam);
        break;
      case SLIDER:
        j = dJointCreateSlider(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetSliderAxis(j, x1[0], x1[1], x1[2]);
        set_limot(j, 0, jp, dJointSetSliderParam);
        break;
      case UNIVERSAL:
        j = dJointCreateUniversal(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetUniversalAnchor(j, a[0], a[1], a[2]);
        dJointSetUniversalAxis1(j, x1[0], x1[1], x1[2]);
        dJointSetUniversalAxis2(j, x2[0], x2[1], x2[2]);
        set_limot(j, 0, jp, dJointSetUniversalParam);
        set_limot(j, 1, jp + 9, dJointSetUniversalParam);
        break;
      case HINGE2:
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
      case AMOTOR: {
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
      case FIXED:
        j = dJointCreateFixed(world, 0);
        dJointAttach(j, B1, B2);
        dJointSetFixed(j);
        dJointSetFixedParam(j, dParamERP, jp[0]);
        dJointSetFixedParam(j, dParamCFM, jp[1]);
        break;
      default: return 2;
    }
    joints[i] = j;
  }

  double* jctl = (double*)calloc((size_t)(nctrl > 0 ? nctrl : 1) * (nj > 0 ? nj : 1) * 3, sizeof(double));
  double* bctl = (double*)calloc((size_t)(nctrl > 0 ? nctrl : 1) * (nb > 0 ? nb : 1) * 6, sizeof(double));
  for (int s = 0; s < nctrl; ++s) {
    if (!rd(in, jctl + (size_t)s * nj * 3, nj * 3)) return 2;
    if (!rd(in, bctl + (size_t)s * nb * 6, nb * 6)) return 2;
  }

  dJointGroupID group = dJointGroupCreate(0);
  dContactGeom cg[16];
  dRandSetSeed(seed);
  for (int s = 0; s < nsteps; ++s) {
    for (int i = 0; i < ng; ++i)
      for (int k = i + 1; k < ng; ++k) {
        const int bi = gbody[i], bk = gbody[k];
        if (bi < 0 && bk < 0) continue;
        if (bi == bk) continue;
        if (bi >= 0 && bk >= 0 && dAreConnectedExcluding(bodies[bi], bodies[bk], dJointTypeContact)) continue;
        const int n = dCollide(geoms[i], geoms[k], maxc, cg, sizeof(dContactGeom));
        const double* S = surf + 12 * (gsurf[i] > gsurf[k] ? gsurf[i] : gsurf[k]);
        for (int c = 0; c < n; ++c) {
          dContact con;
          memset(&con, 0, sizeof(con));
          con.surface.mode = (int)S[0];
          con.surface.mu = S[1];
          con.surface.mu2 = S[2];
          con.surface.bounce = S[3];
          con.surface.bounce_vel = S[4];
          con.surface.soft_erp = S[5];
          con.surface.soft_cfm = S[6];
          con.surface.motion1 = S[7];
          con.surface.motion2 = S[8];
          con.surface.motionN = S[9];
          con.surface.slip1 = S[10];
          con.surface.slip2 = S[11];
          con.geom = cg[c];
          dJointID cj = dJointCreateContact(world, group, &con);
          dJointAttach(cj, bi >= 0 ? bodies[bi] : 0, bk >= 0 ? bodies[bk] : 0);
        }
      }
    if (nctrl > 0) {
      const int cs = s % nctrl;
      const double* jc = jctl + (size_t)cs * nj * 3;
      for (int i = 0; i < nj; ++i) {
        setp_fn setp = stop_setter(jtype[i]);
        if (!setp) continue;
        const double v = jc[3 * i + 2], *jp = jparam + NPARAM * i;
        const double* lp = jtype[i] == AMOTOR ? jp + 5 : jp;
        setp(joints[i], dParamLoStop, isnan(v) ? lp[0] : v);
        setp(joints[i], dParamHiStop, isnan(v) ? lp[1] : v);
      }
      for (int i = 0; i < nj; ++i) {
        const double* t = jc + 3 * i;
        switch (jtype[i]) {
          case HINGE: dJointAddHingeTorque(joints[i], t[0]); break;
          case HINGE2: dJointAddHinge2Torques(joints[i], t[0], t[1]); break;
          case SLIDER: dJointAddSliderForce(joints[i], t[0]); break;
          case UNIVERSAL: dJointAddUniversalTorques(joints[i], t[0], t[1]); break;
          case AMOTOR: dJointAddAMotorTorques(joints[i], t[0], t[1], 0); break;
          default: break;
        }
      }
      const double* bc = bctl + (size_t)cs * nb * 6;
      for (int i = 0; i < nb; ++i) {
        const double* f = bc + 6 * i;
        dBodyAddForce(bodies[i], f[0], f[1], f[2]);
        dBodyAddTorque(bodies[i], f[3], f[4], f[5]);
      }
    }
    const int ok = exact ? dWorldStep(world, dt) : dWorldQuickStep(world, dt);
    if (!ok) { fprintf(stderr, "step %d failed\n", s); return 1; }
    dJointGroupEmpty(group);
  }
  for (int i = 0; i < nb; ++i) {
    const dReal* p = dBodyGetPosition(bodies[i]);
    const dReal* q = dBodyGetQuaternion(bodies[i]);
    const dReal* v = dBodyGetLinearVel(bodies[i]);
    const dReal* w = dBodyGetAngularVel(bodies[i]);
    printf("%.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", p[0], p[1], p[2], q[0],
           q[1], q[2], q[3], v[0], v[1], v[2], w[0], w[1], w[2]);
  }
  dJointGroupDestroy(group);
  dWorldDestroy(world);
  dCloseODE();
  free(surf); free(bodies); free(geoms); free(gbody); free(gsurf); free(joints); free(jtype);
  free(jparam); free(jctl); free(bctl);
  return 0;
}
