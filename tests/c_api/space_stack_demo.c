/*
 * space_stack_demo.c -- a plain ODE program in the shape of ODE's own demos:
 * boxes, spheres and capsules in a hash space over a ground plane, a
 * near-callback that runs dCollide and makes contact joints, auto-disable and
 * damping on, stepped with dWorldQuickStep. It uses only ODE 0.12's public C
 * API: built against the reference (<ode/ode.h>, -DdSINGLE) it runs ODE on the
 * CPU; built against include/ode_gpu.h and linked with libodegpu it runs the
 * same calls with the step and the colliders on the GPU.
 * Input (argv[1]): n_objects n_steps seed.
 * Output: per step "pairs n a b a b ..." (the near-callback's pairs as geom
 * indices) and "contacts n", then one line per body after the last step:
 * pos[3] q[4] enabled. A step that fails prints "step failed" and exits 3.
 */
#include <stdio.h>
#include <stdlib.h>
#ifdef USE_REFERENCE_ODE
#include <ode/ode.h>
#else
#include "ode_gpu.h"
#endif

#define MAX_CONTACTS 4

static dWorldID world;
static dJointGroupID contact_group;
static dGeomID* geoms;
static int n_geoms, n_pairs, n_contacts;
static int pair_buf[4096];

static int geom_index(dGeomID g) {
  for (int i = 0; i < n_geoms; ++i)
    if (geoms[i] == g) return i;
  return -1;
}

static void near_callback(void* data, dGeomID o1, dGeomID o2) {
  (void)data;
  if (n_pairs < 2048) {
    pair_buf[2 * n_pairs] = geom_index(o1);
    pair_buf[2 * n_pairs + 1] = geom_index(o2);
  }
  ++n_pairs;
  dBodyID b1 = dGeomGetBody(o1), b2 = dGeomGetBody(o2);
  if (b1 && b2 && dAreConnectedExcluding(b1, b2, dJointTypeContact)) return;
  dContact contact[MAX_CONTACTS];
  for (int i = 0; i < MAX_CONTACTS; ++i) {
    contact[i].surface.mode = dContactBounce | dContactSoftCFM;
    contact[i].surface.mu = 0.8;
    contact[i].surface.mu2 = 0;
    contact[i].surface.bounce = 0.1;
    contact[i].surface.bounce_vel = 0.1;
    contact[i].surface.soft_cfm = 0.01;
  }
  int n = dCollide(o1, o2, MAX_CONTACTS, &contact[0].geom, sizeof(dContact));
  for (int i = 0; i < n; ++i) {
    dJointID c = dJointCreateContact(world, contact_group, contact + i);
    dJointAttach(c, b1, b2);
  }
  n_contacts += n;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  int n_obj = 0, n_steps = 0;
  unsigned long seed = 0;
  if (sscanf(argv[1], "%d", &n_obj) != 1 || argc < 4 || sscanf(argv[2], "%d", &n_steps) != 1 ||
      sscanf(argv[3], "%lu", &seed) != 1)
    return 2;
  dInitODE2(0);
  world = dWorldCreate();
  dSpaceID space = dHashSpaceCreate(0);
  contact_group = dJointGroupCreate(0);
  dWorldSetGravity(world, 0, 0, -9.81);
  dWorldSetCFM(world, 1e-5);
  dWorldSetAutoDisableFlag(world, 1);
  dWorldSetAutoDisableAverageSamplesCount(world, 10);
  dWorldSetLinearDamping(world, 0.00001);
  dWorldSetAngularDamping(world, 0.005);
  dWorldSetMaxAngularSpeed(world, 200);
  dWorldSetContactMaxCorrectingVel(world, 0.1);
  dWorldSetContactSurfaceLayer(world, 0.001);
  dRandSetSeed(seed);
  geoms = (dGeomID*)calloc(n_obj + 1, sizeof(dGeomID));
  dBodyID* bodies = (dBodyID*)calloc(n_obj, sizeof(dBodyID));
  geoms[0] = dCreatePlane(space, 0, 0, 1, 0);
  n_geoms = 1;
  for (int i = 0; i < n_obj; ++i) {
    bodies[i] = dBodyCreate(world);
    dBodySetPosition(bodies[i], dRandReal() * 2 - 1, dRandReal() * 2 - 1, 0.2 + 0.3 * i);
    dMatrix3 R;
    dRFromAxisAndAngle(R, dRandReal() * 2 - 1, dRandReal() * 2 - 1, dRandReal() * 2 - 1, dRandReal() * 3);
    dBodySetRotation(bodies[i], R);
    dMass m;
    const dReal a = 0.3 + 0.4 * dRandReal(), b = 0.3 + 0.4 * dRandReal(), c = 0.3 + 0.4 * dRandReal();
    switch (i % 3) {
      case 0: geoms[i + 1] = dCreateBox(space, a, b, c); dMassSetBox(&m, 5, a, b, c); break;
      case 1: geoms[i + 1] = dCreateSphere(space, 0.5 * a); dMassSetSphere(&m, 5, 0.5 * a); break;
      default: geoms[i + 1] = dCreateCapsule(space, 0.3 * a, b); dMassSetCapsule(&m, 5, 3, 0.3 * a, b); break;
    }
    dBodySetMass(bodies[i], &m);
    dGeomSetBody(geoms[i + 1], bodies[i]);
    ++n_geoms;
  }
  for (int s = 0; s < n_steps; ++s) {
    n_pairs = n_contacts = 0;
    dSpaceCollide(space, 0, near_callback);
    printf("pairs %d", n_pairs);
    for (int k = 0; k < n_pairs && k < 2048; ++k) printf(" %d %d", pair_buf[2 * k], pair_buf[2 * k + 1]);
    printf("\ncontacts %d\n", n_contacts);
    fflush(stdout);
    if (!dWorldQuickStep(world, 0.01)) {
      printf("step failed\n");
      return 3;
    }
    dJointGroupEmpty(contact_group);
  }
  for (int i = 0; i < n_obj; ++i) {
    const dReal* p = dBodyGetPosition(bodies[i]);
    const dReal* q = dBodyGetQuaternion(bodies[i]);
    printf("%.9g %.9g %.9g %.9g %.9g %.9g %.9g %d\n", p[0], p[1], p[2], q[0], q[1], q[2], q[3],
           dBodyIsEnabled(bodies[i]));
  }
  dJointGroupDestroy(contact_group);
  dSpaceDestroy(space);
  dWorldDestroy(world);
  dCloseODE();
  return 0;
}
