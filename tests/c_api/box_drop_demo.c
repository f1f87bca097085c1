/*
 * box_drop_demo.c -- a plain ODE program (boxes dropped on a plane) that uses
 * only ODE 0.12's public C API. Built against the reference (<ode/ode.h>,
 * -DdSINGLE, linked with the reference library) it runs ODE on the CPU; built
 * against include/ode_gpu.h and linked with libodegpu it runs the same calls
 * on the GPU. Input (text, stdin or argv[1]):
 *   n_boxes n_steps seed
 *   lx ly lz x y z mass I11 I22 I33      (one line per box)
 * Output: one line per body after the last step: pos[3] q[4] lvel[3] avel[3].
 */
#include <stdio.h>
#include <stdlib.h>
#ifdef USE_REFERENCE_ODE
#include <ode/ode.h>
#else
#include "ode_gpu.h"
#endif

int main(int argc, char** argv) {
  FILE* in = argc > 1 ? fopen(argv[1], "r") : stdin;
  int nbox, nsteps;
  unsigned long seed;
  if (!in || fscanf(in, "%d %d %lu", &nbox, &nsteps, &seed) != 3) return 2;
  dInitODE2(0);
  dWorldID world = dWorldCreate();
  dWorldSetGravity(world, 0, 0, -9.81);
  dWorldSetERP(world, 0.2);
  dWorldSetCFM(world, 1e-5);
  dWorldSetQuickStepNumIterations(world, 20);
  dWorldSetQuickStepW(world, 1.3);
  dGeomID* geoms = (dGeomID*)calloc(nbox + 1, sizeof(dGeomID));
  dBodyID* bodies = (dBodyID*)calloc(nbox, sizeof(dBodyID));
  geoms[0] = dCreatePlane(0, 0, 0, 1, 0);
  for (int i = 0; i < nbox; ++i) {
    double lx, ly, lz, x, y, z, m, i11, i22, i33;
    if (fscanf(in, "%lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", &lx, &ly, &lz, &x, &y, &z, &m, &i11, &i22,
               &i33) != 10)
      return 2;
    bodies[i] = dBodyCreate(world);
    dBodySetPosition(bodies[i], x, y, z);
    dMass mass;
    dMassSetParameters(&mass, m, 0, 0, 0, i11, i22, i33, 0, 0, 0);
    dBodySetMass(bodies[i], &mass);
    geoms[i + 1] = dCreateBox(0, lx, ly, lz);
    dGeomSetBody(geoms[i + 1], bodies[i]);
  }
  dJointGroupID contacts = dJointGroupCreate(0);
  dRandSetSeed(seed);
  dContactGeom cg[4];
  for (int s = 0; s < nsteps; ++s) {
    for (int i = 0; i <= nbox; ++i)
      for (int k = i + 1; k <= nbox; ++k) {
        dBodyID b1 = dGeomGetBody(geoms[i]), b2 = dGeomGetBody(geoms[k]);
        if (b1 && b2 && dAreConnectedExcluding(b1, b2, dJointTypeContact)) continue;
        int n = dCollide(geoms[i], geoms[k], 4, cg, sizeof(dContactGeom));
        for (int c = 0; c < n; ++c) {
          dContact con;
          con.surface.mode = dContactApprox1 | dContactSoftERP | dContactSoftCFM;
          con.surface.mu = 0.5;
          con.surface.mu2 = 0;
          con.surface.bounce = 0;
          con.surface.bounce_vel = 0;
          con.surface.soft_erp = 0.2;
          con.surface.soft_cfm = 1e-5;
          con.surface.motion1 = con.surface.motion2 = con.surface.motionN = 0;
          con.surface.slip1 = con.surface.slip2 = 0;
          con.geom = cg[c];
          dJointID j = dJointCreateContact(world, contacts, &con);
          dJointAttach(j, b1, b2);
        }
      }
    if (!dWorldQuickStep(world, 0.01)) { fprintf(stderr, "step %d failed\n", s); return 1; }
    dJointGroupEmpty(contacts);
  }
  for (int i = 0; i < nbox; ++i) {
    const dReal* p = dBodyGetPosition(bodies[i]);
    const dReal* q = dBodyGetQuaternion(bodies[i]);
    const dReal* v = dBodyGetLinearVel(bodies[i]);
    const dReal* w = dBodyGetAngularVel(bodies[i]);
    printf("%.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", p[0], p[1], p[2], q[0],
           q[1], q[2], q[3], v[0], v[1], v[2], w[0], w[1], w[2]);
  }
  dJointGroupDestroy(contacts);
  dWorldDestroy(world);
  dCloseODE();
  return 0;
}
