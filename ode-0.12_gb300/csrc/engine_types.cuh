// engine_types.cuh -- device-resident data layout of a batch of worlds.
//
// Everything is structure-of-arrays indexed by a GLOBAL object index
// (world offset + local index) so that the lanes of the warp owning a world
// read consecutive bodies with coalesced 16-byte loads.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace og {

// Joint types (ODE dJointType values) and surface mode bits (dContact).
enum { J_BALL = 1, J_HINGE = 2, J_SLIDER = 3, J_CONTACT = 4, J_UNIVERSAL = 5, J_HINGE2 = 6, J_FIXED = 7,
       J_AMOTOR = 9 };
enum { AMOTOR_USER = 0, AMOTOR_EULER = 1 };
enum {
  SURF_MU2 = 0x001, SURF_FDIR1 = 0x002, SURF_BOUNCE = 0x004, SURF_SOFT_ERP = 0x008,
  SURF_SOFT_CFM = 0x010, SURF_MOTION1 = 0x020, SURF_MOTION2 = 0x040, SURF_MOTIONN = 0x080,
  SURF_SLIP1 = 0x100, SURF_SLIP2 = 0x200, SURF_APPROX1_1 = 0x1000, SURF_APPROX1_2 = 0x2000
};
// BODY_WOKEN: disabled when the step began and joined by an enabled joint to
// an enabled body, so the step's island walk enables it; it never starts an
// island (ode/src/util.cpp:420-423 skips disabled bodies as starts)
enum { BODY_GYROSCOPIC = 1, BODY_NO_GRAVITY = 2, BODY_WOKEN = 4 };

// Per-world status bits (odegpuBatchStatus).
enum {
  ST_CONTACT_OVERFLOW = 1,   // more contacts than the world's capacity
  ST_ROW_OVERFLOW = 2,       // more constraint rows than the world's capacity
  ST_TOO_LARGE = 4,          // world exceeds the on-chip limits of this kernel
  ST_NONFINITE = 8,          // a body state became NaN/Inf
  ST_HF_ZONE = 32,           // a geom covered more heightfield samples than the collider's buffer
  ST_PAIR_OVERFLOW = 64,     // large world: candidate partners or pairs above capacity
  ST_SOLVE_STALL = 128,      // large world: a bounded wait of the sweep gave up
  ST_LCP_STOP = 256          // dWorldStep: the LCP stopped on a non-positive step (s <= 0)
};

// Row store: 32 words (128 bytes, one cache line) per constraint row.
//   [0..11]  J (scaled by Ad after the setup phase)
//   [12..23] iMJ = invM * J^T
//   [24] c -> b (rhs * Ad)   [25] cfm -> Ad*cfm   [26] lo  [27] hi
//   [28] findex (world row index or -1, int bits)  [29] b1  [30] b2  [31] joint
// The optional unscaled dump (StepOptions::dbg_rows) keeps J in [0..11], Ad in
// [12], that erp in [13], rhs in [24], cfm/h in [25] and words 26..31 as above.
constexpr int kRowWords = 32;
constexpr int kRowC = 24, kRowCfm = 25, kRowLo = 26, kRowHi = 27, kRowFindex = 28;
constexpr int kRowB1 = 29, kRowB2 = 30, kRowJoint = 31;
constexpr int kDbgAd = 12, kDbgErp = 13;

struct DevSurface {
  int mode;
  float mu, mu2, bounce, bounce_vel, soft_erp, soft_cfm, motion1, motion2, motionN, slip1, slip2;
};

struct DevLimot {
  float vel, fmax, lostop, histop, fudge, normal_cfm, stop_erp, stop_cfm, bounce;
};

// A persistent (non-contact) joint after dJointAttach and its setters.
struct DevJoint {
  int type, b1, b2, reverse;    // b1/b2 world-local, b2 = -1 for the environment
  float anchor1[4], anchor2[4], axis1[4], axis2[4];
  float qrel[4];                // hinge, slider, fixed: qrel; universal: qrel1
  union {
    float v1[4];                // hinge2
    float offset[4];            // slider, fixed: body-1 centre relative to body 2
  };
  union {
    float v2[4];                // hinge2
    float qrel2[4];             // universal
  };
  float erp, cfm, c0, s0, susp_erp, susp_cfm;   // erp / cfm: ball and fixed
  DevLimot lm1, lm2;
  // angular motor (ode/src/joints/amotor.h): lm1 / lm2 / lm3 drive axes 0 / 1 / 2
  DevLimot lm3;
  int am_num, am_mode, am_rel[3];
  float am_axis[3][4];          // axes in the frame rel selects (0 world, 1 body 1, 2 body 2)
  float am_ref1[4], am_ref2[4]; // Euler mode reference vectors
  float am_angle[3];            // user mode angles (dJointSetAMotorAngle)
};

// A contact produced by the narrowphase and turned into a contact joint.
struct DevContact {
  float pos[3], depth;
  float normal[3];
  int surface;
  int b1, b2, reverse;          // attach result: b2 = -1 for the environment
  int geoms;                    // world-local pair (g1 | g2 << 8) of the collider call and, for a
                                // heightfield contact, how it arose << 16; -1 unknown
};

// A heightfield (dGeomHeightfieldDataBuild* + placeable dCreateHeightfield)
// with the caches of dxHeightfieldData::SetData (ode/src/heightfield.cpp:107-143).
struct DevHeightfield {
  int nx, nz, wrap, h_off;             // samples; wrap mode; first sample in the sample array
  float width, depth, scale, offset, thickness;
  float sw, sd, inv_sw, inv_sd, zx, half_w, half_d;
  float pos[3], pad;
  float R[12];                         // placement, 3x4 row-major
};

// Static description of one world inside the batch.
struct WorldDesc {
  int body_off, nb, geom_off, ng, joint_off, njp;
  int contact_off, contact_cap;
  int row_off, row_cap;
  int padj_off;                 // persistent adjacency (CSR) offset
  int fwd_scratch;              // slot of the forward sweep's global scratch (a row capacity
                                // above what the warp's shared memory holds), or -1
  int max_contacts;
  int iterations;
  float gravity[3], erp, cfm, sor_w, max_vel, min_depth, dt;
  int hf_ws_side;               // samples per axis of the world's heightfield workspace (0: none)
  long long hf_ws;              // its byte offset in BatchDev::hf_ws
};

// dxStepBody options of a body (ode/src/objects.h:38-47 flags, util.cpp:255-360):
// record [0] = (flags as int bits, maximum angular speed, linear damping scale,
// linear threshold squared), [1] = (angular scale, angular threshold squared,
// finite rotation axis x, y), [2] = (axis z, 0, 0, 0)
constexpr int kStepRec = 3;
constexpr int kStepFiniteRot = 1, kStepFiniteAxis = 2, kStepLinDamp = 4, kStepAngDamp = 8, kStepMaxAng = 16;

struct BatchDev {
  int n_worlds;
  const WorldDesc* world;
  unsigned* seed;               // [n_worlds] dRand state
  int* status;                  // [n_worlds] ST_* bits
  int* ncontacts;               // [n_worlds] contacts of the last step
  int* nrows;                   // [n_worlds] rows of the last step
  int* nislands;                // [n_worlds] islands of the last step

  // bodies
  float4 *pos, *q, *lvel, *avel;       // [nb_total]
  float *mass, *invMass;               // [nb_total]
  float *I, *invI;                     // [nb_total][9] body frame
  int* bflags;                         // [nb_total]
  // per-body dxStepBody options, kStepRec float4 per body (kStep* above);
  // null when no body of the batch uses one
  const float4* bstep;
  float* invIw;                        // [nb_total][12] scratch: world-frame invI
  float4 *facc, *tacc;                 // [nb_total] scratch accumulators

  // geoms
  const int* gtype;                    // [ng_total]
  const int* gbody;                    // world-local body or -1
  const float4* gparam;                // class parameters
  const float* gbound;                 // bounding radius (INFINITY for planes)
  const float4* gpos;                  // static placement (geoms without body)
  const int* gsurf;
  const DevSurface* surfaces;
  const DevHeightfield* hfs;           // heightfields (geom param x = index)
  const float* hf_heights;             // their samples, x fastest

  // persistent joints and their adjacency
  const DevJoint* joints;              // [nj_total]
  const int* padj_start;               // [nb_total + n_worlds]: per-world CSR starts
  const int* padj;                     // persistent joint ordinals, newest first

  // per-step controls
  int n_ctrl_steps;
  const float* joint_torque;           // [S][nj_total][2]
  const float* body_force;             // [S][nb_total][6]
  const float* joint_stop;             // [S][nj_total] limot1 lostop = histop (NaN: the joint's own)
  int step_counter_base;

  // per-step scratch (capacity-sized per world)
  DevContact* contacts;                // [contact_cap_total]
  float* rows;                         // [row_cap_total][32]
  float4* sweep;                       // per world (row_cap + 32) x 8 float4: the rows of the
                                       // current reshuffle round in execution order, quad-major
  unsigned char* fwd_scratch;          // row-indexed SOR arrays of worlds with a large row capacity
  unsigned char* hf_ws;                // heightfield zone workspaces of worlds whose geoms need one
  int* jlist;                          // [njp + contact_cap per world] island order
  int* adj;                            // [2 * (njp + contact_cap) per world]
  int* adj_start;                      // [nb_total + n_worlds]
  int* island_jstart;                  // [nb_total + n_worlds]
  int* island_rstart;                  // [nb_total + n_worlds]
  int* jrow;                           // [njp + contact_cap per world] first row per joint
  int* jm;                             // [...] rows per joint
};

}  // namespace og
