// engine_internal.hpp -- internal interface between the ODE-compatible API
// layer (ode_api.cpp) and the device engine (engine.cu).
#pragma once
#include <vector>
#include "engine_types.cuh"
#include "collide.cuh"
#include "host_setup.hpp"

namespace og {

// FP32 copy of the setter results: the fields every joint has, plus the
// per-type ones that share storage in DevJoint (hinge2 v1/v2, slider / fixed
// offset, universal qrel2).
inline void pack_joint_geometry(int type, const og_host::HJoint& H, DevJoint& J) {
  for (int k = 0; k < 4; ++k) {
    J.anchor1[k] = (float)H.anchor1[k]; J.anchor2[k] = (float)H.anchor2[k];
    J.axis1[k] = (float)H.axis1[k]; J.axis2[k] = (float)H.axis2[k];
    J.qrel[k] = (float)H.qrel[k];
    if (type == J_HINGE2) { J.v1[k] = (float)H.v1[k]; J.v2[k] = (float)H.v2[k]; }
    else if (type == J_SLIDER || type == J_FIXED) J.offset[k] = (float)H.offset[k];
    else if (type == J_UNIVERSAL) J.qrel2[k] = (float)H.qrel2[k];
  }
  J.c0 = (float)H.c0; J.s0 = (float)H.s0;
  if (type == J_AMOTOR) {
    J.am_num = H.am_num;
    J.am_mode = H.am_mode;
    for (int i = 0; i < 3; ++i) {
      J.am_rel[i] = H.am_rel[i];
      J.am_angle[i] = (float)H.am_angle[i];
      for (int k = 0; k < 4; ++k) J.am_axis[i][k] = (float)H.am_axis[i][k];
    }
    for (int k = 0; k < 4; ++k) { J.am_ref1[k] = (float)H.am_ref1[k]; J.am_ref2[k] = (float)H.am_ref2[k]; }
  }
}

// One world as the ODE API layer hands it to the device, in ODE's creation
// order, with complete per-body joint lists (newest attachment first).
struct HostWorld {
  WorldDesc desc;                     // offsets 0; nb, njp, contact_cap, row_cap set
  std::vector<float4> pos, q, lvel, avel, facc, tacc;
  std::vector<float> mass, invMass, I, invI;
  std::vector<int> flags;
  std::vector<float4> bstep;          // dxStepBody options (kStepRec per body), empty when none used
  std::vector<DevJoint> joints;       // persistent joints with bodies attached
  std::vector<DevContact> contacts;   // contact joints, creation order
  std::vector<DevSurface> surfaces;   // one per contact
  std::vector<int> padj_start, padj;  // full body lists (ordinals: joint, njp + contact)
  unsigned seed = 0;
  int status = 0;
  bool want_feedback = false;         // compute joint feedback in ctx_step
  bool exact = false;                 // dWorldStep instead of dWorldQuickStep
  std::vector<float> feedback;        // out: [njp][12] persistent joints (f1 t1 f2 t2)
  std::vector<float> contact_feedback;// out: [contacts][12]
};

struct WorldCtx;
WorldCtx* ctx_create(int device);
void ctx_destroy(WorldCtx* c);
// Uploads hw, runs one world step on the GPU, writes the new body state (pos,
// q, lvel, avel) and the RNG state back into hw. Returns 0 or an ODEGPU_E code.
int ctx_step(WorldCtx* c, HostWorld& hw);
// The colliders' closest points of two segments (host side of a
// __host__ __device__ routine), for dClosestLineSegmentPoints.
void closest_segment_points_host(const float* a1, const float* a2, const float* b1, const float* b2, float* cp1,
                                 float* cp2);
// The box-box collider on the host, for dBoxBox (at most 8 contacts).
int box_box_host(const float* p1, const float* R1, const float* side1, const float* p2, const float* R2,
                 const float* side2, float* normal, float* depth, int* code, unsigned flags, Contact* out);
// One dCollide on the GPU. Returns the contact count (<= 8) or a negative code.
int collide_pair_gpu(const GeomView& a, const GeomView& b, unsigned flags, Contact* out);
// Heightfields for the ODE API: the dxHeightfieldData caches, the device copy
// of the samples, and dCollide(heightfield, g) with the field first.
DevHeightfield make_dev_heightfield(int nx, int nz, double width, double depth, double scale, double offset,
                                   double thickness, int wrap, const double* pos, const double* R9, int h_off);
int upload_heights(const std::vector<float>& h, float** dev);
void free_heights(float* dev);
int collide_hf_gpu(const DevHeightfield& H, const float* d_heights, const GeomView& g, unsigned flags, Contact* out);

}  // namespace og
