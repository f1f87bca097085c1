/*
 * odegpu_scene.h -- flat, seeded description of a batch of independent ODE worlds.
 *
 * One description feeds three consumers that must agree object-for-object:
 *   - libodegpu (the CUDA path, FP32 on the device),
 *   - the CPU oracle under oracle/ (FP64 restatement, test infrastructure),
 *   - the harness that drives the reference ODE 0.12 through its public API.
 *
 * Creation order is part of the contract because ODE's row order is emergent:
 * bodies, geoms and joints are created in array order, so the reference's
 * prepend-on-create lists (ode/src/ode.cpp:62-68 addObjectToList, :272 in
 * dBodyCreate; ode/src/joints/joint.cpp:56 in the joint constructor; body joint
 * lists prepended in dJointAttach, ode/src/ode.cpp:1379-1392) come out newest
 * first. Contacts are generated in the canonical pair order described at
 * odegpuCanonicalPairs below.
 *
 * All per-object indices are WORLD-LOCAL (0-based within the world); -1 means
 * "static environment" for a body index.
 */
#ifndef ODEGPU_SCENE_H
#define ODEGPU_SCENE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Geom classes. Numbering follows ODE's dGeomClass enum
 * (include/ode/collision.h:881-890) for the classes on this path. */
enum {
  ODEGPU_GEOM_SPHERE = 0,
  ODEGPU_GEOM_BOX = 1,
  ODEGPU_GEOM_CAPSULE = 2,
  ODEGPU_GEOM_CYLINDER = 3,     /* flat-ended; param radius, length along local z */
  ODEGPU_GEOM_PLANE = 4,
  ODEGPU_GEOM_RAY = 5,          /* queries only (dCollide, odegpuBatchRayCast);
                                   a scene may not hold one */
  ODEGPU_GEOM_HEIGHTFIELD = 9
};

/* Persistent joint types (values are ODE's dJointType, include/ode/common.h). */
enum {
  ODEGPU_JOINT_BALL = 1,
  ODEGPU_JOINT_HINGE = 2,
  ODEGPU_JOINT_SLIDER = 3,
  ODEGPU_JOINT_CONTACT = 4,
  ODEGPU_JOINT_UNIVERSAL = 5,
  ODEGPU_JOINT_HINGE2 = 6,
  ODEGPU_JOINT_FIXED = 7,
  ODEGPU_JOINT_AMOTOR = 9
};

/* dContact surface mode bits (include/ode/contact.h:33-49). */
enum {
  ODEGPU_CONTACT_MU2 = 0x001,
  ODEGPU_CONTACT_FDIR1 = 0x002,
  ODEGPU_CONTACT_BOUNCE = 0x004,
  ODEGPU_CONTACT_SOFT_ERP = 0x008,
  ODEGPU_CONTACT_SOFT_CFM = 0x010,
  ODEGPU_CONTACT_MOTION1 = 0x020,
  ODEGPU_CONTACT_MOTION2 = 0x040,
  ODEGPU_CONTACT_MOTIONN = 0x080,
  ODEGPU_CONTACT_SLIP1 = 0x100,
  ODEGPU_CONTACT_SLIP2 = 0x200,
  ODEGPU_CONTACT_APPROX1_1 = 0x1000,
  ODEGPU_CONTACT_APPROX1_2 = 0x2000,
  ODEGPU_CONTACT_APPROX1 = 0x3000
};

/* Body flags (subset of ODE's dxBodyFlags, ode/src/objects.h:38-52). */
enum { ODEGPU_BODY_GYROSCOPIC = 1, ODEGPU_BODY_NO_GRAVITY = 2 };

/* Surface parameters: same fields and meaning as dSurfaceParameters
 * (include/ode/contact.h:52-65). */
typedef struct odegpuSurface {
  int mode;
  double mu, mu2, bounce, bounce_vel, soft_erp, soft_cfm;
  double motion1, motion2, motionN, slip1, slip2;
} odegpuSurface;

/* Per-world stepping parameters (dWorldSet* in include/ode/objects.h). */
typedef struct odegpuWorldParams {
  double gravity[3];
  double erp, cfm;          /* dWorldSetERP / dWorldSetCFM, set explicitly   */
  int iterations;           /* dWorldSetQuickStepNumIterations               */
  double sor_w;             /* dWorldSetQuickStepW                           */
  double max_vel;           /* dWorldSetContactMaxCorrectingVel              */
  double min_depth;         /* dWorldSetContactSurfaceLayer                  */
  double dt;                /* step size handed to dWorldQuickStep           */
  int max_contacts;         /* flags & 0xffff handed to dCollide, 1..16      */
  unsigned int seed;        /* dRandSetSeed before the world's first step    */
} odegpuWorldParams;

/* Number of doubles per joint in odegpuScene.joint_param. Layout:
 *   ball, fixed: [0]=erp [1]=cfm
 *   hinge, slider: [0..8] = limot {lostop, histop, vel, fmax, fudge, bounce,
 *                           cfm, stop_erp, stop_cfm}
 *   universal: [0..8] limot1, [9..17] limot2
 *   hinge2: [0..8] limot1, [9..17] limot2, [18] susp_erp, [19] susp_cfm
 *   amotor: [0] number of axes, [1] mode (0 user, 1 Euler), [2..4] rel of
 *           axes 0..2 (0 global, 1 body 1, 2 body 2), [5..13] limot of axis 0,
 *           [14..22] axis 1, [23..31] axis 2, [32..34] user-mode angles
 * (dxJointLimitMotor fields, ode/src/joints/joint.h:160-170). The geometry
 * setters used per type: ball and universal take joint_anchor; hinge,
 * hinge2, slider and universal take joint_axis1; hinge2 and universal take
 * joint_axis2; the fixed joint takes the bodies' placement at creation
 * (dJointSetFixed); the amotor's axes 0, 1, 2 (world frame, as
 * dJointSetAMotorAxis takes them) are joint_anchor, joint_axis1,
 * joint_axis2, set in the order mode, number of axes, axes, parameters,
 * angles. */
#define ODEGPU_JOINT_NPARAM 36
/* Number of doubles per geom in odegpuScene.geom_param:
 *   sphere [0]=r; box [0..2]=side; capsule [0]=r [1]=length;
 *   cylinder [0]=r [1]=length; plane [0..3]=a,b,c,d (normalised as
 *   dCreatePlane does); heightfield [0]=index into heightfields; ray
 *   [0]=length (queries only). */
#define ODEGPU_GEOM_NPARAM 4

typedef struct odegpuHeightfield {
  int nx, nz;              /* samples along local x (width) and z (depth)    */
  double width, depth;     /* extent along local x and z                     */
  double scale, offset, thickness;
  int wrap;
  const double* heights;   /* nz * nx samples, row-major in z then x         */
  double pos[3];           /* placement of the heightfield geom              */
  double R[9];             /* row-major rotation of the heightfield geom     */
} odegpuHeightfield;

typedef struct odegpuScene {
  int n_worlds;
  /* prefix offsets, each of length n_worlds+1 */
  const int* body_off;
  const int* geom_off;
  const int* joint_off;
  const odegpuWorldParams* world;      /* [n_worlds] */

  /* bodies: global arrays indexed by body_off[w] + local index */
  const double* body_pos;    /* [nb][3] */
  const double* body_q;      /* [nb][4] (w,x,y,z), normalised on load        */
  const double* body_lvel;   /* [nb][3] */
  const double* body_avel;   /* [nb][3] */
  const double* body_mass;   /* [nb]    */
  const double* body_I;      /* [nb][9] row-major body-frame inertia         */
  const int* body_flags;     /* [nb]    ODEGPU_BODY_*                         */

  /* geoms */
  const int* geom_type;      /* [ng] */
  const int* geom_body;      /* [ng] world-local body index or -1 (static)   */
  const double* geom_param;  /* [ng][ODEGPU_GEOM_NPARAM]                      */
  const int* geom_surface;   /* [ng] index into surfaces                      */
  const odegpuSurface* surfaces; int n_surfaces;
  const odegpuHeightfield* heightfields; int n_heightfields; /* geom_param[0] of a
                                   heightfield geom holds its index here     */

  /* persistent joints */
  const int* joint_type;     /* [nj] ODEGPU_JOINT_*                           */
  const int* joint_body;     /* [nj][2] world-local (b1, b2), b2 may be -1    */
  const double* joint_anchor;/* [nj][3] world-frame anchor                    */
  const double* joint_axis1; /* [nj][3] */
  const double* joint_axis2; /* [nj][3] */
  const double* joint_param; /* [nj][ODEGPU_JOINT_NPARAM]                     */

  /* optional per-step controls (NULL = none); n_ctrl_steps steps are stored and
   * step s uses row (s % n_ctrl_steps). */
  int n_ctrl_steps;
  const double* joint_torque;  /* [n_ctrl_steps][nj][2]: hinge torque in [0]
                                  (dJointAddHingeTorque), hinge2 and universal
                                  torque1/torque2 in [0]/[1]
                                  (dJointAddHinge2Torques,
                                  dJointAddUniversalTorques), slider force in
                                  [0] (dJointAddSliderForce), amotor torques
                                  about axes 0 and 1 in [0]/[1]
                                  (dJointAddAMotorTorques with 0 about axis 2) */
  const double* body_force;    /* [n_ctrl_steps][nb][6]: force, torque        */
  const double* joint_stop;    /* [n_ctrl_steps][nj]: before the step, limot1
                                  lostop = histop of a hinge, hinge2 or
                                  universal joint (an angle) or of a slider (a
                                  position) to this value (dJointSet*Param
                                  with dParamLoStop, dParamHiStop); NaN leaves
                                  the joint's own stops from joint_param    */
} odegpuScene;

/*
 * Canonical pair order (replaces dSpaceCollide's enumeration, which depends on
 * space internals, ode/src/collision_space.cpp:247-266): within a world, geoms
 * are visited in index order and dCollide(g_i, g_j, max_contacts) is called for
 * every i < j, skipping pairs where both geoms are static or both sit on the
 * same body (the same early-outs dCollide applies, ode/src/collision_kernel.cpp
 * :307-311), and pairs whose bodies are joined by a persistent (non-contact)
 * joint (the dAreConnectedExcluding(b1, b2, dJointTypeContact) test of ODE's
 * demo near-callbacks, ode/src/ode.cpp:1529-1537, e.g. ode/demo/
 * demo_boxstack.cpp:140). Each returned contact becomes a contact joint attached to
 * (body(g_i), body(g_j)), in contact order. This file only documents the rule;
 * every consumer implements it.
 */

#ifdef __cplusplus
}
#endif
#endif
