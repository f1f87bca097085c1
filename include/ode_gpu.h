/*
 * ode_gpu.h -- ODE 0.12's C API for the contact-generation + QuickStep path,
 * exported by libodegpu with dReal = float (ODE's dSINGLE). A program written
 * against <ode/ode.h> that uses only these entry points links against
 * libodegpu instead of libode; the step runs on the GPU through the same
 * kernels as the batched API (odegpu.h). Each declaration cites the reference
 * declaration it replaces (include/ode/<file>:<line>).
 *
 * Differences from the reference, all deliberate:
 *  - dWorldQuickStep runs one world per call on the GPU (a launch plus the
 *    host<->device copies of that world); for many worlds use odegpu.h.
 *  - dCollide runs the collider on the GPU, one launch per call.
 *  - Errors never abort the process: dWorldQuickStep returns 0 and
 *    odegpuGetLastError() says why (ODE aborts on debug asserts).
 *  - joints with dJointSetFeedback get f1 t1 (and f2 t2 with a second body)
 *    after each dWorldQuickStep, as ODE's quickstep fills them.
 *  - A world of up to 64 bodies whose joints and contacts cannot need more
 *    than 1024 constraint rows steps in one on-chip kernel per phase; a
 *    larger world (up to 65536 bodies) steps through the large-world
 *    pipeline of odegpu.h with the caller's contacts, joint feedback
 *    included. dWorldStep is available on the first path only: for a larger
 *    world it returns 0.
 *  - Spaces, geom placement, auto-disable and the other bookkeeping run on
 *    the host as in ODE (same pair order, same island order); moved
 *    callbacks run after the whole step rather than body by body, and a
 *    heightfield's height callback is sampled once when the data is built.
 *  - Not built: trimesh, convex, and
 *    the LMotor, PR, PU, piston and plane-2D joints.
 */
#ifndef ODE_GPU_H
#define ODE_GPU_H

#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef float dReal;
typedef dReal dVector3[4];
typedef dReal dVector4[4];
typedef dReal dMatrix3[4 * 3];
typedef dReal dQuaternion[4];

typedef struct dxWorld* dWorldID;
typedef struct dxBody* dBodyID;
typedef struct dxJoint* dJointID;
typedef struct dxJointGroup* dJointGroupID;
typedef struct dxGeom* dGeomID;
typedef struct dxSpace* dSpaceID;

/* include/ode/mass.h:88-92 */
typedef struct dMass {
  dReal mass;
  dVector3 c;
  dMatrix3 I;
} dMass;

/* include/ode/contact.h:33-49 */
enum {
  dContactMu2 = 0x001, dContactFDir1 = 0x002, dContactBounce = 0x004,
  dContactSoftERP = 0x008, dContactSoftCFM = 0x010, dContactMotion1 = 0x020,
  dContactMotion2 = 0x040, dContactMotionN = 0x080, dContactSlip1 = 0x100,
  dContactSlip2 = 0x200, dContactApprox0 = 0x0000, dContactApprox1_1 = 0x1000,
  dContactApprox1_2 = 0x2000, dContactApprox1 = 0x3000
};

/* include/ode/contact.h:52-65 */
typedef struct dSurfaceParameters {
  int mode;
  dReal mu;
  dReal mu2, bounce, bounce_vel, soft_erp, soft_cfm, motion1, motion2, motionN, slip1, slip2;
} dSurfaceParameters;

/* include/ode/contact.h:82-88 */
typedef struct dContactGeom {
  dVector3 pos;
  dVector3 normal;
  dReal depth;
  dGeomID g1, g2;
  int side1, side2;
} dContactGeom;

/* include/ode/contact.h:93-97 */
typedef struct dContact {
  dSurfaceParameters surface;
  dContactGeom geom;
  dVector3 fdir1;
} dContact;

/* include/ode/common.h:368-373 */
typedef struct dJointFeedback {
  dVector3 f1, t1, f2, t2;
} dJointFeedback;

/* include/ode/collision.h:881-899 */
enum { dSphereClass = 0, dBoxClass, dCapsuleClass, dCylinderClass, dPlaneClass,
       dRayClass, dConvexClass, dGeomTransformClass, dTriMeshClass, dHeightfieldClass,
       dFirstSpaceClass, dSimpleSpaceClass = dFirstSpaceClass, dHashSpaceClass,
       dSweepAndPruneSpaceClass, dQuadTreeSpaceClass, dLastSpaceClass = dQuadTreeSpaceClass };

/* include/ode/common.h:252-258 */
typedef enum { dJointTypeNone = 0, dJointTypeBall, dJointTypeHinge, dJointTypeSlider,
               dJointTypeContact, dJointTypeUniversal, dJointTypeHinge2, dJointTypeFixed,
               dJointTypeNull, dJointTypeAMotor } dJointType;
/* angular motor modes (include/ode/common.h:360-363) */
enum { dAMotorUser = 0, dAMotorEuler = 1 };

/* include/ode/common.h:305-354 */
enum {
  dParamLoStop = 0, dParamHiStop, dParamVel, dParamFMax, dParamFudgeFactor, dParamBounce,
  dParamCFM, dParamStopERP, dParamStopCFM, dParamSuspensionERP, dParamSuspensionCFM,
  dParamERP,
  dParamGroup = 0x100,
  dParamLoStop2 = 0x100, dParamHiStop2, dParamVel2, dParamFMax2, dParamFudgeFactor2,
  dParamBounce2, dParamCFM2, dParamStopERP2, dParamStopCFM2
};

/* init: include/ode/odeinit.h:95, :119, :227 */
void dInitODE(void);
int dInitODE2(unsigned int uiInitFlags);
void dCloseODE(void);
/* include/ode/odeinit.h:177-204 and objects.h:157-289: per-thread data and
 * step working memory are the GPU path's own, so these accept and return 1 */
int dAllocateODEDataForThread(unsigned int uiAllocateFlags);             /* odeinit.h:177 */
void dCleanupODEAllDataForThread(void);                                  /* odeinit.h:204 */
typedef struct {
  unsigned struct_size;
  float reserve_factor;
  unsigned reserve_minimum;
} dWorldStepReserveInfo;                                                 /* objects.h:201-207 */
typedef struct {
  unsigned struct_size;
  void* (*alloc_block)(size_t block_size);
  void* (*shrink_block)(void* block_pointer, size_t block_current_size, size_t block_smaller_size);
  void (*free_block)(void* block_pointer, size_t block_current_size);
} dWorldStepMemoryFunctionsInfo;                                         /* objects.h:256-263 */
#define dWORLDSTEP_RESERVEFACTOR_DEFAULT 1.2f
#define dWORLDSTEP_RESERVESIZE_DEFAULT 65536U
int dWorldUseSharedWorkingMemory(dWorldID w, dWorldID from_world);      /* objects.h:157 */
void dWorldCleanupWorkingMemory(dWorldID w);                             /* objects.h:180 */
int dWorldSetStepMemoryReservationPolicy(dWorldID w, const dWorldStepReserveInfo* policyinfo);  /* objects.h:234 */
int dWorldSetStepMemoryManager(dWorldID w, const dWorldStepMemoryFunctionsInfo* memfuncs);       /* objects.h:289 */
const char* dGetConfiguration(void);                                     /* common.h:404 */
int dCheckConfiguration(const char* token);                              /* common.h:414 */

/* world: include/ode/objects.h */
dWorldID dWorldCreate(void);                                        /* :54  */
void dWorldDestroy(dWorldID w);                                     /* :66  */
void dWorldSetGravity(dWorldID w, dReal x, dReal y, dReal z);       /* :77  */
void dWorldGetGravity(dWorldID w, dVector3 gravity);                /* :84  */
void dWorldSetERP(dWorldID w, dReal erp);                           /* :94  */
dReal dWorldGetERP(dWorldID w);                                     /* :101 */
void dWorldSetCFM(dWorldID w, dReal cfm);                           /* :111 */
dReal dWorldGetCFM(dWorldID w);                                     /* :118 */
int dWorldQuickStep(dWorldID w, dReal stepsize);                    /* :352 */
void dWorldImpulseToForce(dWorldID w, dReal stepsize, dReal ix, dReal iy, dReal iz,
                          dVector3 force);                            /* :369 */
/* The exact stepper (dense LCP per island, Dantzig pivoting) on the GPU. */
int dWorldStep(dWorldID w, dReal stepsize);                         /* :309 */
void dWorldSetQuickStepNumIterations(dWorldID w, int num);          /* :385 */
int dWorldGetQuickStepNumIterations(dWorldID w);                    /* :394 */
void dWorldSetQuickStepW(dWorldID w, dReal over_relaxation);        /* :401 */
dReal dWorldGetQuickStepW(dWorldID w);                              /* :408 */
void dWorldSetContactMaxCorrectingVel(dWorldID w, dReal vel);       /* :420 */
dReal dWorldGetContactMaxCorrectingVel(dWorldID w);                 /* :427 */
void dWorldSetContactSurfaceLayer(dWorldID w, dReal depth);         /* :440 */
dReal dWorldGetContactSurfaceLayer(dWorldID w);                     /* :447 */
/* Damping and the angular speed cap, applied by the step's body update on
 * the GPU (ode/src/util.cpp:255-360) */
dReal dWorldGetLinearDampingThreshold(dWorldID w);                  /* :635 */
void dWorldSetLinearDampingThreshold(dWorldID w, dReal threshold);  /* :643 */
dReal dWorldGetAngularDampingThreshold(dWorldID w);                 /* :649 */
void dWorldSetAngularDampingThreshold(dWorldID w, dReal threshold); /* :657 */
dReal dWorldGetLinearDamping(dWorldID w);                           /* :663 */
void dWorldSetLinearDamping(dWorldID w, dReal scale);               /* :671 */
dReal dWorldGetAngularDamping(dWorldID w);                          /* :677 */
void dWorldSetAngularDamping(dWorldID w, dReal scale);              /* :685 */
void dWorldSetDamping(dWorldID w, dReal linear_scale, dReal angular_scale);  /* :693 */
dReal dWorldGetMaxAngularSpeed(dWorldID w);                         /* :702 */
void dWorldSetMaxAngularSpeed(dWorldID w, dReal max_speed);         /* :710 */
/* Auto-disable, checked on the host at the start of every step
 * (ode/src/util.cpp:98-230); a disabled body is left out of the step until an
 * enabled joint connects it to an enabled body. dWorldGetAutoDisableFlag
 * returns ODE 0.12's raw flag bit (16) when set. */
dReal dWorldGetAutoDisableLinearThreshold(dWorldID w);              /* :487 */
void dWorldSetAutoDisableLinearThreshold(dWorldID w, dReal linear_threshold);    /* :494 */
dReal dWorldGetAutoDisableAngularThreshold(dWorldID w);             /* :501 */
void dWorldSetAutoDisableAngularThreshold(dWorldID w, dReal angular_threshold);  /* :508 */
int dWorldGetAutoDisableAverageSamplesCount(dWorldID w);            /* :543 */
void dWorldSetAutoDisableAverageSamplesCount(dWorldID w, unsigned int average_samples_count);  /* :551 */
int dWorldGetAutoDisableSteps(dWorldID w);                          /* :558 */
void dWorldSetAutoDisableSteps(dWorldID w, int steps);              /* :565 */
dReal dWorldGetAutoDisableTime(dWorldID w);                         /* :572 */
void dWorldSetAutoDisableTime(dWorldID w, dReal time);              /* :579 */
int dWorldGetAutoDisableFlag(dWorldID w);                           /* :586 */
void dWorldSetAutoDisableFlag(dWorldID w, int do_auto_disable);     /* :593 */
dReal dBodyGetAutoDisableLinearThreshold(dBodyID b);                /* :753 */
void dBodySetAutoDisableLinearThreshold(dBodyID b, dReal linear_average_threshold);   /* :760 */
dReal dBodyGetAutoDisableAngularThreshold(dBodyID b);               /* :767 */
void dBodySetAutoDisableAngularThreshold(dBodyID b, dReal angular_average_threshold); /* :774 */
int dBodyGetAutoDisableAverageSamplesCount(dBodyID b);              /* :781 */
void dBodySetAutoDisableAverageSamplesCount(dBodyID b, unsigned int average_samples_count);  /* :788 */
int dBodyGetAutoDisableSteps(dBodyID b);                            /* :796 */
void dBodySetAutoDisableSteps(dBodyID b, int steps);                /* :803 */
dReal dBodyGetAutoDisableTime(dBodyID b);                           /* :810 */
void dBodySetAutoDisableTime(dBodyID b, dReal time);                /* :817 */
int dBodyGetAutoDisableFlag(dBodyID b);                             /* :824 */
void dBodySetAutoDisableFlag(dBodyID b, int do_auto_disable);       /* :831 */
void dBodySetAutoDisableDefaults(dBodyID b);                        /* :839 */

/* bodies: include/ode/objects.h */
dBodyID dBodyCreate(dWorldID w);                                    /* :856 */
void dBodyDestroy(dBodyID b);                                       /* :866 */
void dBodySetPosition(dBodyID b, dReal x, dReal y, dReal z);        /* :890 */
void dBodySetRotation(dBodyID b, const dMatrix3 R);                 /* :900 */
void dBodySetQuaternion(dBodyID b, const dQuaternion q);            /* :910 */
void dBodySetLinearVel(dBodyID b, dReal x, dReal y, dReal z);       /* :916 */
void dBodySetAngularVel(dBodyID b, dReal x, dReal y, dReal z);      /* :922 */
const dReal* dBodyGetPosition(dBodyID b);                           /* :933 */
const dReal* dBodyGetRotation(dBodyID b);                           /* :951 */
const dReal* dBodyGetQuaternion(dBodyID b);                         /* :969 */
const dReal* dBodyGetLinearVel(dBodyID b);                          /* :986 */
const dReal* dBodyGetAngularVel(dBodyID b);                         /* :992 */
void dBodySetMass(dBodyID b, const dMass* mass);                    /* :998 */
void dBodyGetMass(dBodyID b, dMass* mass);                          /* :1004 */
void dBodyAddForce(dBodyID b, dReal fx, dReal fy, dReal fz);        /* :1010 */
void dBodyAddTorque(dBodyID b, dReal fx, dReal fy, dReal fz);       /* :1016 */
const dReal* dBodyGetForce(dBodyID b);                              /* :1064 */
const dReal* dBodyGetTorque(dBodyID b);                             /* :1075 */
void dBodySetForce(dBodyID b, dReal x, dReal y, dReal z);           /* :1085 */
void dBodySetTorque(dBodyID b, dReal x, dReal y, dReal z);          /* :1095 */
void dBodyAddRelForce(dBodyID b, dReal fx, dReal fy, dReal fz);     /* :1022 */
void dBodyAddRelTorque(dBodyID b, dReal fx, dReal fy, dReal fz);    /* :1028 */
void dBodyAddForceAtPos(dBodyID b, dReal fx, dReal fy, dReal fz,
                        dReal px, dReal py, dReal pz);              /* :1034 */
void dBodyAddForceAtRelPos(dBodyID b, dReal fx, dReal fy, dReal fz,
                           dReal px, dReal py, dReal pz);           /* :1040 */
void dBodyAddRelForceAtPos(dBodyID b, dReal fx, dReal fy, dReal fz,
                           dReal px, dReal py, dReal pz);           /* :1046 */
void dBodyAddRelForceAtRelPos(dBodyID b, dReal fx, dReal fy, dReal fz,
                              dReal px, dReal py, dReal pz);        /* :1052 */
void dBodyGetRelPointPos(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result);  /* :1102 */
void dBodyGetRelPointVel(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result);  /* :1113 */
void dBodyGetPointVel(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result);     /* :1125 */
void dBodyGetPosRelPoint(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result);  /* :1139 */
void dBodyVectorToWorld(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result);   /* :1150 */
void dBodyVectorFromWorld(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result); /* :1161 */
void dBodySetData(dBodyID b, void* data);                           /* :873 */
void* dBodyGetData(dBodyID b);                                      /* :880 */
/* A step moves the enabled bodies and those an enabled joint connects to
 * them (enabling them, as ODE's island walk does); other disabled bodies keep
 * their state and their accumulated forces. */
void dBodySetDynamic(dBodyID b);                                    /* :1241 */
void dBodySetKinematic(dBodyID b);                                  /* :1255 */
int dBodyIsKinematic(dBodyID b);                                    /* :1262 */
void dBodyEnable(dBodyID b);                                        /* :1269 */
void dBodyDisable(dBodyID b);                                       /* :1278 */
int dBodyIsEnabled(dBodyID b);                                      /* :1285 */
void dBodySetFiniteRotationMode(dBodyID b, int mode);               /* :1184 */
void dBodySetFiniteRotationAxis(dBodyID b, dReal x, dReal y, dReal z);  /* :1202 */
int dBodyGetFiniteRotationMode(dBodyID b);                          /* :1209 */
void dBodyGetFiniteRotationAxis(dBodyID b, dVector3 result);        /* :1216 */
/* The moved callback runs after each step for every body, in island order,
 * once all bodies hold their new state (ODE runs it as each body is stepped). */
void dBodySetMovedCallback(dBodyID b, void (*callback)(dBodyID));   /* :1316 */
dGeomID dBodyGetFirstGeom(dBodyID b);                               /* :1328 */
dGeomID dBodyGetNextGeom(dGeomID g);                                /* :1338 */
void dBodySetDampingDefaults(dBodyID b);                            /* :1345 */
dReal dBodyGetLinearDamping(dBodyID b);                             /* :1351 */
void dBodySetLinearDamping(dBodyID b, dReal scale);                 /* :1361 */
dReal dBodyGetAngularDamping(dBodyID b);                            /* :1369 */
void dBodySetAngularDamping(dBodyID b, dReal scale);                /* :1379 */
void dBodySetDamping(dBodyID b, dReal linear_scale, dReal angular_scale);  /* :1388 */
dReal dBodyGetLinearDampingThreshold(dBodyID b);                    /* :1394 */
void dBodySetLinearDampingThreshold(dBodyID b, dReal threshold);    /* :1402 */
dReal dBodyGetAngularDampingThreshold(dBodyID b);                   /* :1408 */
void dBodySetAngularDampingThreshold(dBodyID b, dReal threshold);   /* :1416 */
dReal dBodyGetMaxAngularSpeed(dBodyID b);                           /* :1423 */
void dBodySetMaxAngularSpeed(dBodyID b, dReal max_speed);           /* :1433 */
int dBodyGetNumJoints(dBodyID b);                                   /* :1223 */
void dBodyCopyPosition(dBodyID b, dVector3 pos);                    /* :943 */
void dBodyCopyRotation(dBodyID b, dMatrix3 R);                      /* :961 */
void dBodyCopyQuaternion(dBodyID b, dQuaternion quat);              /* :979 */
dWorldID dBodyGetWorld(dBodyID b);                                  /* :848 */
dJointID dBodyGetJoint(dBodyID b, int index);                       /* :1231 */
void dBodySetGravityMode(dBodyID b, int mode);                      /* :1294 */
int dBodyGetGravityMode(dBodyID b);                                 /* :1301 */
void dBodySetGyroscopicMode(dBodyID b, int enabled);                /* :1458 */
int dBodyGetGyroscopicMode(dBodyID b);                              /* :1444 */

/* joints: include/ode/objects.h */
dJointID dJointCreateBall(dWorldID w, dJointGroupID g);                  /* :1538 */
dJointID dJointCreateHinge(dWorldID w, dJointGroupID g);                 /* :1546 */
dJointID dJointCreateContact(dWorldID w, dJointGroupID g, const dContact* c); /* :1562 */
dJointID dJointCreateHinge2(dWorldID w, dJointGroupID g);                /* :1570 */
dJointID dJointCreateSlider(dWorldID w, dJointGroupID g);                /* :1554 */
dJointID dJointCreateUniversal(dWorldID w, dJointGroupID g);             /* :1578 */
dJointID dJointCreateFixed(dWorldID w, dJointGroupID g);                 /* :1611 */
dJointID dJointCreateNull(dWorldID w, dJointGroupID g);                  /* :1613 */
void dJointDestroy(dJointID j);                                          /* :1647 */
void dJointSetData(dJointID j, void* data);                              /* :1722 */
void* dJointGetData(dJointID j);                                         /* :1728 */
dJointGroupID dJointGroupCreate(int max_size);                           /* :1655 */
void dJointGroupDestroy(dJointGroupID g);                                /* :1663 */
void dJointGroupEmpty(dJointGroupID g);                                  /* :1672 */
void dJointAttach(dJointID j, dBodyID body1, dBodyID body2);             /* :1693 */
dJointType dJointGetType(dJointID j);                                    /* :1749 */
dBodyID dJointGetBody(dJointID j, int index);                            /* :1761 */
void dJointEnable(dJointID j);                                            /* :1700 */
void dJointDisable(dJointID j);                                           /* :1709 */
int dJointIsEnabled(dJointID j);                                          /* :1716 */
int dJointGetNumBodies(dJointID j);                                      /* :1678 */
dJointID dConnectingJoint(dBodyID b1, dBodyID b2);                       /* :2940 */
int dConnectingJointList(dBodyID b1, dBodyID b2, dJointID* out);         /* :2945 */
void dJointSetFeedback(dJointID j, dJointFeedback* f);                   /* :1770 */
dJointFeedback* dJointGetFeedback(dJointID j);                           /* :1776 */
void dJointSetBallAnchor(dJointID j, dReal x, dReal y, dReal z);         /* :1785 */
void dJointSetBallAnchor2(dJointID j, dReal x, dReal y, dReal z);        /* :1791 */
void dJointSetBallParam(dJointID j, int parameter, dReal value);         /* :1797 */
void dJointGetBallAnchor(dJointID j, dVector3 result);                   /* :2351 */
void dJointGetBallAnchor2(dJointID j, dVector3 result);                  /* :2363 */
dReal dJointGetBallParam(dJointID j, int parameter);                     /* :2369 */
void dJointSetHingeAnchor(dJointID j, dReal x, dReal y, dReal z);        /* :1803 */
void dJointSetHingeAxis(dJointID j, dReal x, dReal y, dReal z);          /* :1811 */
void dJointSetHingeAnchorDelta(dJointID j, dReal x, dReal y, dReal z, dReal dx, dReal dy, dReal dz);  /* :1805 */
void dJointSetHingeAxisOffset(dJointID j, dReal x, dReal y, dReal z, dReal angle);  /* :1841 */
void dJointGetHingeAnchor(dJointID j, dVector3 result);                  /* :2378 */
void dJointGetHingeAnchor2(dJointID j, dVector3 result);                 /* :2388 */
void dJointGetHingeAxis(dJointID j, dVector3 result);                    /* :2394 */
void dJointSetHingeParam(dJointID j, int parameter, dReal value);        /* :1847 */
dReal dJointGetHingeParam(dJointID j, int parameter);                    /* :2400 */
dReal dJointGetHingeAngle(dJointID j);                                   /* :2414 */
dReal dJointGetHingeAngleRate(dJointID j);                               /* :2420 */
void dJointAddHingeTorque(dJointID j, dReal torque);                     /* :1857 */
void dJointSetHinge2Anchor(dJointID j, dReal x, dReal y, dReal z);       /* :1890 */
void dJointSetHinge2Axis1(dJointID j, dReal x, dReal y, dReal z);        /* :1896 */
void dJointSetHinge2Axis2(dJointID j, dReal x, dReal y, dReal z);        /* :1902 */
void dJointGetHinge2Anchor(dJointID j, dVector3 result);                 /* :2459 */
void dJointGetHinge2Anchor2(dJointID j, dVector3 result);                /* :2469 */
void dJointGetHinge2Axis1(dJointID j, dVector3 result);                  /* :2475 */
void dJointGetHinge2Axis2(dJointID j, dVector3 result);                  /* :2481 */
void dJointSetHinge2Param(dJointID j, int parameter, dReal value);       /* :1908 */
dReal dJointGetHinge2Param(dJointID j, int parameter);                   /* :2487 */
void dJointAddHinge2Torques(dJointID j, dReal torque1, dReal torque2);   /* :1916 */
dReal dJointGetHinge2Angle1(dJointID j);                                 /* :2493 */
dReal dJointGetHinge2Angle1Rate(dJointID j);                             /* :2499 */
dReal dJointGetHinge2Angle2Rate(dJointID j);                             /* :2505 */
void dJointSetSliderAxis(dJointID j, dReal x, dReal y, dReal z);         /* :1863 */
void dJointSetSliderAxisDelta(dJointID j, dReal x, dReal y, dReal z, dReal dx, dReal dy, dReal dz);  /* :1868 */
void dJointSetSliderParam(dJointID j, int parameter, dReal value);       /* :1874 */
void dJointAddSliderForce(dJointID j, dReal force);                      /* :1884 */
dReal dJointGetSliderPosition(dJointID j);                               /* :2433 */
dReal dJointGetSliderPositionRate(dJointID j);                           /* :2439 */
void dJointGetSliderAxis(dJointID j, dVector3 result);                   /* :2445 */
dReal dJointGetSliderParam(dJointID j, int parameter);                   /* :2451 */
void dJointSetUniversalAnchor(dJointID j, dReal x, dReal y, dReal z);    /* :1922 */
void dJointSetUniversalAxis1(dJointID j, dReal x, dReal y, dReal z);     /* :1928 */
void dJointSetUniversalAxis2(dJointID j, dReal x, dReal y, dReal z);     /* :1973 */
void dJointSetUniversalAxis1Offset(dJointID j, dReal x, dReal y, dReal z, dReal offset1, dReal offset2);  /* :1966 */
void dJointSetUniversalAxis2Offset(dJointID j, dReal x, dReal y, dReal z, dReal offset1, dReal offset2);  /* :2013 */
void dJointSetUniversalParam(dJointID j, int parameter, dReal value);    /* :2020 */
void dJointAddUniversalTorques(dJointID j, dReal torque1, dReal torque2);/* :2028 */
void dJointGetUniversalAnchor(dJointID j, dVector3 result);              /* :2513 */
void dJointGetUniversalAnchor2(dJointID j, dVector3 result);             /* :2528 */
void dJointGetUniversalAxis1(dJointID j, dVector3 result);               /* :2534 */
void dJointGetUniversalAxis2(dJointID j, dVector3 result);               /* :2540 */
dReal dJointGetUniversalParam(dJointID j, int parameter);                /* :2547 */
void dJointGetUniversalAngles(dJointID j, dReal* angle1, dReal* angle2); /* :2560 */
dReal dJointGetUniversalAngle1(dJointID j);                              /* :2566 */
dReal dJointGetUniversalAngle2(dJointID j);                              /* :2572 */
dReal dJointGetUniversalAngle1Rate(dJointID j);                          /* :2578 */
dReal dJointGetUniversalAngle2Rate(dJointID j);                          /* :2584 */
void dJointSetFixed(dJointID j);                                         /* :2247 */
void dJointSetFixedParam(dJointID j, int parameter, dReal value);        /* :2254 */
dReal dJointGetFixedParam(dJointID j, int parameter);                    /* :2934 */
dJointID dJointCreateAMotor(dWorldID w, dJointGroupID g);                /* :1621 */
void dJointSetAMotorNumAxes(dJointID j, int num);                        /* :2261 */
void dJointSetAMotorAxis(dJointID j, int anum, int rel, dReal x, dReal y, dReal z); /* :2267 */
void dJointSetAMotorAngle(dJointID j, int anum, dReal angle);            /* :2279 */
void dJointSetAMotorParam(dJointID j, int parameter, dReal value);       /* :2285 */
void dJointSetAMotorMode(dJointID j, int mode);                          /* :2291 */
void dJointAddAMotorTorques(dJointID j, dReal torque1, dReal torque2, dReal torque3); /* :2301 */
int dJointGetAMotorNumAxes(dJointID j);                                  /* :2840 */
void dJointGetAMotorAxis(dJointID j, int anum, dVector3 result);         /* :2851 */
int dJointGetAMotorAxisRel(dJointID j, int anum);                        /* :2869 */
dReal dJointGetAMotorAngle(dJointID j, int anum);                        /* :2879 */
dReal dJointGetAMotorAngleRate(dJointID j, int anum);                    /* :2889, 0 (unimplemented in ODE 0.12) */
dReal dJointGetAMotorParam(dJointID j, int parameter);                   /* :2895 */
int dJointGetAMotorMode(dJointID j);                                     /* :2910 */
int dAreConnectedExcluding(dBodyID b1, dBodyID b2, int joint_type);      /* :2968 */
int dAreConnected(dBodyID b1, dBodyID b2);                               /* :2953 */

/* mass: include/ode/mass.h */
void dMassSetZero(dMass* m);                                             /* :45 */
void dMassSetParameters(dMass* m, dReal themass, dReal cgx, dReal cgy, dReal cgz,
                        dReal I11, dReal I22, dReal I33, dReal I12, dReal I13,
                        dReal I23);                                      /* :47 */
void dMassSetSphere(dMass* m, dReal density, dReal radius);              /* :52 */
void dMassSetSphereTotal(dMass* m, dReal total_mass, dReal radius);      /* :53 */
void dMassSetBox(dMass* m, dReal density, dReal lx, dReal ly, dReal lz); /* :65 */
void dMassSetBoxTotal(dMass* m, dReal total_mass, dReal lx, dReal ly, dReal lz); /* :67 */
void dMassSetCapsule(dMass* m, dReal density, int direction, dReal radius, dReal length);       /* :55 */
void dMassSetCapsuleTotal(dMass* m, dReal total_mass, int direction, dReal radius, dReal length); /* :57 */
void dMassSetCylinder(dMass* m, dReal density, int direction, dReal radius, dReal length);      /* :60 */
void dMassSetCylinderTotal(dMass* m, dReal total_mass, int direction, dReal radius, dReal length); /* :62 */
void dMassAdjust(dMass* m, dReal newmass);                               /* :74 */
int dMassCheck(const dMass* m);                                          /* :43 */
void dMassTranslate(dMass* m, dReal x, dReal y, dReal z);                /* :76 */
void dMassRotate(dMass* m, const dMatrix3 R);                            /* :78 */
void dMassAdd(dMass* a, const dMass* b);                                 /* :80 */
void dMassSetCappedCylinder(dMass* m, dReal density, int direction, dReal radius, dReal length);  /* :84 */
void dMassSetCappedCylinderTotal(dMass* m, dReal total_mass, int direction, dReal radius,
                                 dReal length);                                               /* :85 */

/* RNG: include/ode/misc.h */
int dTestRand(void);                                                     /* :37 */
unsigned long dRand(void);                                               /* :42 */
unsigned long dRandGetSeed(void);                                        /* :45 */
void dRandSetSeed(unsigned long s);                                      /* :46 */
int dRandInt(int n);                                                     /* :51 */
dReal dRandReal(void);                                                   /* :54 */

/* rotation and vector utilities: include/ode/rotation.h, include/ode/odemath.h
 * (FP32, the reference's operation order) */
void dRSetIdentity(dMatrix3 R);                                          /* rotation.h:34 */
void dRFromAxisAndAngle(dMatrix3 R, dReal ax, dReal ay, dReal az, dReal angle);   /* :36 */
void dRFromEulerAngles(dMatrix3 R, dReal phi, dReal theta, dReal psi);  /* :39 */
void dRFrom2Axes(dMatrix3 R, dReal ax, dReal ay, dReal az, dReal bx, dReal by, dReal bz);  /* :41 */
void dRFromZAxis(dMatrix3 R, dReal ax, dReal ay, dReal az);             /* :44 */
void dQSetIdentity(dQuaternion q);                                       /* :46 */
void dQFromAxisAndAngle(dQuaternion q, dReal ax, dReal ay, dReal az, dReal angle);  /* :48 */
void dQMultiply0(dQuaternion qa, const dQuaternion qb, const dQuaternion qc);  /* :53 */
void dQMultiply1(dQuaternion qa, const dQuaternion qb, const dQuaternion qc);  /* :55 */
void dQMultiply2(dQuaternion qa, const dQuaternion qb, const dQuaternion qc);  /* :57 */
void dQMultiply3(dQuaternion qa, const dQuaternion qb, const dQuaternion qc);  /* :59 */
void dRfromQ(dMatrix3 R, const dQuaternion q);                           /* :61 */
void dQfromR(dQuaternion q, const dMatrix3 R);                           /* :62 */
void dDQfromW(dReal dq[4], const dVector3 w, const dQuaternion q);      /* :63 */
int dSafeNormalize3(dVector3 a);                                         /* odemath.h:424 */
int dSafeNormalize4(dVector4 a);                                         /* :425 */
void dNormalize3(dVector3 a);                                            /* :426 */
void dNormalize4(dVector4 a);                                            /* :427 */
void dPlaneSpace(const dVector3 n, dVector3 p, dVector3 q);              /* :462 */
void dOrthogonalizeR(dMatrix3 m);                                        /* :464 */
/* include/ode/misc.h: matrices with rows padded to a multiple of 4 */
void dPrintMatrix(const dReal* A, int n, int m, const char* fmt, FILE* f);  /* misc.h:61 */
void dMakeRandomVector(dReal* A, int n, dReal range);                    /* misc.h:65 */
void dMakeRandomMatrix(dReal* A, int n, int m, dReal range);             /* :68 */
void dClearUpperTriangle(dReal* A, int n);                               /* :71 */
dReal dMaxDifference(const dReal* A, const dReal* B, int n, int m);      /* :74 */
dReal dMaxDifferenceLowerTriangle(const dReal* A, const dReal* B, int n);  /* :78 */

/* collision: include/ode/collision.h */
int dCollide(dGeomID o1, dGeomID o2, int flags, dContactGeom* contact, int skip); /* :795 */
/* A caller's collider for a class pair runs on the host in place of the
 * built-in one; dCloseODE drops the overrides. */
typedef int dColliderFn(dGeomID o1, dGeomID o2, int flags, dContactGeom* contact, int skip);  /* :1488 */
void dSetColliderOverride(int i, int j, dColliderFn* fn);                /* :1514 */
/* User geom classes (at most four): their colliders, boxes and box tests are
 * the caller's host functions. */
typedef void dGetAABBFn(dGeomID g, dReal aabb[6]);                       /* :1487 */
typedef dColliderFn* dGetColliderFnFn(int num);                          /* :1490 */
typedef void dGeomDtorFn(dGeomID o);                                     /* :1491 */
typedef int dAABBTestFn(dGeomID o1, dGeomID o2, dReal aabb[6]);          /* :1492 */
typedef struct dGeomClass {
  int bytes;
  dGetColliderFnFn* collider;
  dGetAABBFn* aabb;
  dAABBTestFn* aabb_test;
  dGeomDtorFn* dtor;
} dGeomClass;                                                            /* :1494-1500 */
int dCreateGeomClass(const dGeomClass* classptr);                        /* :1502 */
void* dGeomGetClassData(dGeomID g);                                      /* :1503 */
dGeomID dCreateGeom(int classnum);                                       /* :1504 */
/* Geom transforms: the wrapped geom collides at the transform's pose. */
dGeomID dCreateGeomTransform(dSpaceID space);                            /* :1086 */
void dGeomTransformSetGeom(dGeomID g, dGeomID obj);                      /* :1087 */
dGeomID dGeomTransformGetGeom(dGeomID g);                                /* :1088 */
void dGeomTransformSetCleanup(dGeomID g, int mode);                      /* :1089 */
int dGeomTransformGetCleanup(dGeomID g);                                 /* :1090 */
void dGeomTransformSetInfo(dGeomID g, int mode);                         /* :1091 */
int dGeomTransformGetInfo(dGeomID g);                                    /* :1092 */
dGeomID dCreateSphere(dSpaceID space, dReal radius);                     /* :924 */
dGeomID dCreateBox(dSpaceID space, dReal lx, dReal ly, dReal lz);        /* :1002 */
dGeomID dCreatePlane(dSpaceID space, dReal a, dReal b, dReal c, dReal d); /* :1046 */
dGeomID dCreateCapsule(dSpaceID space, dReal radius, dReal length);      /* :1051 */
/* Flat-ended cylinders: dCollide with sphere, box, plane, ray and heightfield;
 * cylinder-cylinder and capsule-cylinder return no contacts, as in a reference
 * build without libccd. */
dGeomID dCreateCylinder(dSpaceID space, dReal radius, dReal length);     /* :1063 */
void dGeomCylinderSetParams(dGeomID cylinder, dReal radius, dReal length);   /* :1064 */
void dGeomCylinderGetParams(dGeomID cylinder, dReal* radius, dReal* length); /* :1065 */
/* Rays: dCollide of a ray with a sphere, box, capsule, plane or heightfield
 * returns at most one contact whose depth is the distance along the ray. */
dGeomID dCreateRay(dSpaceID space, dReal length);                        /* :1067 */
void dGeomRaySetLength(dGeomID ray, dReal length);                       /* :1068 */
dReal dGeomRayGetLength(dGeomID ray);                                    /* :1069 */
void dGeomRaySet(dGeomID ray, dReal px, dReal py, dReal pz, dReal dx, dReal dy, dReal dz);  /* :1070 */
void dGeomRayGet(dGeomID ray, dVector3 start, dVector3 dir);             /* :1072 */
void dGeomRaySetParams(dGeomID g, int FirstContact, int BackfaceCull);   /* :1079 */
void dGeomRayGetParams(dGeomID g, int* FirstContact, int* BackfaceCull); /* :1080 */
void dGeomRaySetClosestHit(dGeomID g, int closestHit);                   /* :1081 */
int dGeomRayGetClosestHit(dGeomID g);                                    /* :1082 */
/* Heightfields: the samples are copied when the data is built (ODE can keep
 * a reference to the caller's array when bCopyHeightData is 0). */
typedef struct dxHeightfieldData* dHeightfieldDataID;                   /* collision.h:1101 */
dGeomID dCreateHeightfield(dSpaceID space, dHeightfieldDataID data, int bPlaceable);  /* :1144 */
dHeightfieldDataID dGeomHeightfieldDataCreate(void);                    /* :1160 */
void dGeomHeightfieldDataDestroy(dHeightfieldDataID d);                 /* :1171 */
void dGeomHeightfieldDataBuildSingle(dHeightfieldDataID d, const float* pHeightData, int bCopyHeightData,
                                     dReal width, dReal depth, int widthSamples, int depthSamples,
                                     dReal scale, dReal offset, dReal thickness, int bWrap);  /* :1361 */
void dGeomHeightfieldDataBuildByte(dHeightfieldDataID d, const unsigned char* pHeightData, int bCopyHeightData,
                                   dReal width, dReal depth, int widthSamples, int depthSamples,
                                   dReal scale, dReal offset, dReal thickness, int bWrap);  /* :1263 */
void dGeomHeightfieldDataBuildShort(dHeightfieldDataID d, const short* pHeightData, int bCopyHeightData,
                                    dReal width, dReal depth, int widthSamples, int depthSamples,
                                    dReal scale, dReal offset, dReal thickness, int bWrap);  /* :1311 */
void dGeomHeightfieldDataSetBounds(dHeightfieldDataID d, dReal minHeight, dReal maxHeight);  /* :1433 */
typedef dReal dHeightfieldGetHeight(void* p_user_data, int x, int z);  /* collision.h:1121 */
void dGeomHeightfieldDataBuildCallback(dHeightfieldDataID d, void* pUserData, dHeightfieldGetHeight* pCallback,
                                       dReal width, dReal depth, int widthSamples, int depthSamples,
                                       dReal scale, dReal offset, dReal thickness, int bWrap);  /* :1215 */
void dGeomHeightfieldSetHeightfieldData(dGeomID g, dHeightfieldDataID d);   /* :1447 */
dHeightfieldDataID dGeomHeightfieldGetHeightfieldData(dGeomID g);          /* :1459 */
void dGeomHeightfieldDataBuildDouble(dHeightfieldDataID d, const double* pHeightData, int bCopyHeightData,
                                     dReal width, dReal depth, int widthSamples, int depthSamples,
                                     dReal scale, dReal offset, dReal thickness, int bWrap);  /* :1411 */
void dGeomDestroy(dGeomID g);                                            /* :68  */
void dGeomSetData(dGeomID g, void* data);                                /* :78  */
void* dGeomGetData(dGeomID g);                                           /* :87  */
/* Placement. A geom on a body follows the body; with an offset it sits at
 * body + offset, and dGeomGetPosition/Rotation and dCollide read that pose.
 * dGeomSetBody(g, 0) keeps the geom where it was; dBodyDestroy detaches the
 * body's geoms the same way. */
void dGeomSetBody(dGeomID g, dBodyID body);                              /* :108 */
dBodyID dGeomGetBody(dGeomID g);                                         /* :117 */
void dGeomSetPosition(dGeomID g, dReal x, dReal y, dReal z);             /* :134 */
void dGeomSetRotation(dGeomID g, const dMatrix3 R);                      /* :149 */
void dGeomSetQuaternion(dGeomID g, const dQuaternion Q);                 /* :165 */
const dReal* dGeomGetPosition(dGeomID g);                                /* :184 */
void dGeomCopyPosition(dGeomID g, dVector3 pos);                         /* :194 */
const dReal* dGeomGetRotation(dGeomID g);                                /* :213 */
void dGeomCopyRotation(dGeomID g, dMatrix3 R);                           /* :229 */
void dGeomGetQuaternion(dGeomID g, dQuaternion result);                  /* :245 */
void dGeomGetAABB(dGeomID g, dReal aabb[6]);                             /* :264 */
int dGeomIsSpace(dGeomID g);                                             /* :273 */
void dInfiniteAABB(dGeomID g, dReal aabb[6]);                            /* :1481 */
enum { dGeomCommonControlClass = 0, dGeomColliderControlClass = 1 };     /* :412-415 */
int dGeomLowLevelControl(dGeomID g, int controlClass, int controlCode, void* dataValue, int* dataSize);  /* :460 */
void dClosestLineSegmentPoints(const dVector3 a1, const dVector3 a2, const dVector3 b1, const dVector3 b2,
                               dVector3 cp1, dVector3 cp2);              /* :1466 */
int dBoxBox(const dVector3 p1, const dMatrix3 R1, const dVector3 side1, const dVector3 p2, const dMatrix3 R2,
            const dVector3 side2, dVector3 normal, dReal* depth, int* return_code, int flags,
            dContactGeom* contact, int skip);                           /* :1475 */
int dBoxTouchesBox(const dVector3 p1, const dMatrix3 R1, const dVector3 side1, const dVector3 p2,
                   const dMatrix3 R2, const dVector3 side2);             /* :1470 */
dSpaceID dGeomGetSpace(dGeomID g);                                       /* :283 */
int dGeomGetClass(dGeomID g);                                            /* :310 */
/* Category / collide bits and the enabled flag steer a space's pair search;
 * dCollide reads none of them. */
void dGeomSetCategoryBits(dGeomID g, unsigned long bits);                /* :325 */
void dGeomSetCollideBits(dGeomID g, unsigned long bits);                 /* :340 */
unsigned long dGeomGetCategoryBits(dGeomID g);                           /* :351 */
unsigned long dGeomGetCollideBits(dGeomID g);                            /* :362 */
void dGeomEnable(dGeomID g);                                             /* :377 */
void dGeomDisable(dGeomID g);                                            /* :392 */
int dGeomIsEnabled(dGeomID g);                                           /* :408 */
void dGeomGetRelPointPos(dGeomID g, dReal px, dReal py, dReal pz, dVector3 result);    /* :472 */
void dGeomGetPosRelPoint(dGeomID g, dReal px, dReal py, dReal pz, dVector3 result);    /* :490 */
void dGeomVectorToWorld(dGeomID g, dReal px, dReal py, dReal pz, dVector3 result);     /* :505 */
void dGeomVectorFromWorld(dGeomID g, dReal px, dReal py, dReal pz, dVector3 result);   /* :520 */
/* Offsets from the body: a geom without a body ignores the setters. */
void dGeomSetOffsetPosition(dGeomID g, dReal x, dReal y, dReal z);       /* :545 */
void dGeomSetOffsetRotation(dGeomID g, const dMatrix3 R);                /* :561 */
void dGeomSetOffsetQuaternion(dGeomID g, const dQuaternion Q);           /* :577 */
void dGeomSetOffsetWorldPosition(dGeomID g, dReal x, dReal y, dReal z);  /* :596 */
void dGeomSetOffsetWorldRotation(dGeomID g, const dMatrix3 R);           /* :613 */
void dGeomSetOffsetWorldQuaternion(dGeomID g, const dQuaternion Q);      /* :630 */
void dGeomClearOffset(dGeomID g);                                        /* :646 */
int dGeomIsOffset(dGeomID g);                                            /* :664 */
const dReal* dGeomGetOffsetPosition(dGeomID g);                          /* :680 */
void dGeomCopyOffsetPosition(dGeomID g, dVector3 pos);                   /* :693 */
const dReal* dGeomGetOffsetRotation(dGeomID g);                          /* :710 */
void dGeomCopyOffsetRotation(dGeomID g, dMatrix3 R);                     /* :724 */
void dGeomGetOffsetQuaternion(dGeomID g, dQuaternion result);            /* :737 */
/* Spaces: include/ode/collision_space.h. Simple and hash spaces enumerate
 * candidate pairs on the host in ODE's order (a geom that moves goes to the
 * front of its space's list, as do the geoms of every body a step moves, in
 * the step's island order), so a near-callback sees the pairs ODE would pass. */
typedef void dNearCallback(void* data, dGeomID o1, dGeomID o2);         /* collision_space.h:49 */
dSpaceID dSimpleSpaceCreate(dSpaceID space);                             /* :52 */
dSpaceID dHashSpaceCreate(dSpaceID space);                               /* :53 */
/* A quadtree over x and y. As in ODE 0.12, dSpaceGetGeom does not enumerate
 * it (returns 0), its box stays infinite, and destroying it does not destroy
 * its geoms (here they are released from it). */
dSpaceID dQuadTreeSpaceCreate(dSpaceID space, const dVector3 Center, const dVector3 Extents, int Depth);  /* :54 */
/* Sweep and prune along the first axis of axisorder (collision_space.h:56-66) */
enum { dSAP_AXES_XYZ = 0 | (1 << 2) | (2 << 4), dSAP_AXES_XZY = 0 | (2 << 2) | (1 << 4),
       dSAP_AXES_YXZ = 1 | (0 << 2) | (2 << 4), dSAP_AXES_YZX = 1 | (2 << 2) | (0 << 4),
       dSAP_AXES_ZXY = 2 | (0 << 2) | (1 << 4), dSAP_AXES_ZYX = 2 | (1 << 2) | (0 << 4) };
dSpaceID dSweepAndPruneSpaceCreate(dSpaceID space, int axisorder);       /* :66 */
void dSpaceDestroy(dSpaceID space);                                      /* :70 */
void dHashSpaceSetLevels(dSpaceID space, int minlevel, int maxlevel);    /* :72 */
void dHashSpaceGetLevels(dSpaceID space, int* minlevel, int* maxlevel);  /* :73 */
void dSpaceSetCleanup(dSpaceID space, int mode);                         /* :75 */
int dSpaceGetCleanup(dSpaceID space);                                    /* :76 */
void dSpaceSetSublevel(dSpaceID space, int sublevel);                    /* :100 */
int dSpaceGetSublevel(dSpaceID space);                                   /* :114 */
void dSpaceSetManualCleanup(dSpaceID space, int mode);                   /* :133 */
int dSpaceGetManualCleanup(dSpaceID space);                              /* :147 */
void dSpaceAdd(dSpaceID space, dGeomID g);                               /* :149 */
void dSpaceRemove(dSpaceID space, dGeomID g);                            /* :150 */
int dSpaceQuery(dSpaceID space, dGeomID g);                              /* :151 */
void dSpaceClean(dSpaceID space);                                        /* :152 */
int dSpaceGetNumGeoms(dSpaceID space);                                   /* :153 */
dGeomID dSpaceGetGeom(dSpaceID space, int i);                            /* :154 */
int dSpaceGetClass(dSpaceID space);                                      /* :176 */
void dSpaceCollide(dSpaceID space, void* data, dNearCallback* callback); /* collision.h:825 */
void dSpaceCollide2(dGeomID space1, dGeomID space2, void* data, dNearCallback* callback);  /* collision.h:868 */
/* class parameters and point depths */
void dGeomSphereSetRadius(dGeomID g, dReal radius);                      /* :936 */
dReal dGeomSphereGetRadius(dGeomID g);                                   /* :947 */
dReal dGeomSpherePointDepth(dGeomID g, dReal x, dReal y, dReal z);       /* :964 */
void dGeomBoxSetLengths(dGeomID g, dReal lx, dReal ly, dReal lz);        /* :1016 */
void dGeomBoxGetLengths(dGeomID g, dVector3 result);                     /* :1028 */
dReal dGeomBoxPointDepth(dGeomID g, dReal x, dReal y, dReal z);          /* :1043 */
void dGeomPlaneSetParams(dGeomID g, dReal a, dReal b, dReal c, dReal d); /* :1047 */
void dGeomPlaneGetParams(dGeomID g, dVector4 result);                    /* :1048 */
dReal dGeomPlanePointDepth(dGeomID g, dReal x, dReal y, dReal z);        /* :1049 */
void dGeomCapsuleSetParams(dGeomID g, dReal radius, dReal length);       /* :1052 */
void dGeomCapsuleGetParams(dGeomID g, dReal* radius, dReal* length);     /* :1053 */
dReal dGeomCapsulePointDepth(dGeomID g, dReal x, dReal y, dReal z);      /* :1054 */

#ifdef __cplusplus
}
#endif
#endif
