// ode_api.cpp -- ODE 0.12's C API (include/ode_gpu.h) over the CUDA path.
//
// Object model: worlds own bodies and persistent joints in creation order;
// joint groups own contact joints; every attachment gets a sequence number so
// that each body's joint list can be produced in ODE's order (dJointAttach
// prepends, ode/src/ode.cpp:1379-1392). dWorldQuickStep packs the world and
// runs one step of the device kernel (engine_internal.hpp); no step math runs
// on the host. Setter arithmetic (anchors, axes, inertia inverse) is host FP64
// as in host_setup.hpp.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "ode_gpu.h"
#include "odegpu.h"
#include "engine_internal.hpp"
#include "host_setup.hpp"

using og::DevContact;
using og::DevJoint;
using og::DevSurface;

struct dxJoint;
struct dxGeom;

struct dxBody {
  dxWorld* world;
  dReal pos[4], q[4], R[12], lvel[4], avel[4], facc[4], tacc[4];
  dMass mass;
  double invI[9];
  double invMass;
  int flags;   // ODEGPU_BODY_*
  void* data;  // dBodySetData
  dxGeom* geom;   // the body's geoms, newest attached first (dxGeom::bodyAdd)
  // dxStepBody options (ode/src/objects.h:38-47, :118-147): og::kStep* flags,
  // the angular speed cap, damping scales and squared thresholds, and the
  // finite rotation axis (normalised, or zero)
  int step_flags;
  dReal max_angular_speed, lin_scale, lin_thr, ang_scale, ang_thr;
  dReal frot_axis[4];
  void (*moved_callback)(dxBody*);   // dBodySetMovedCallback
  int disabled;                      // dBodyDisable, or auto-disabled
  // auto-disable (ode/src/objects.h dxAutoDisable, util.cpp:98-230): the
  // parameters, the idle countdowns and the velocity sample ring
  int auto_disable, adis_steps, adis_stepsleft, avg_ready;
  unsigned adis_samples, avg_counter;
  dReal adis_time, adis_lin_thr, adis_ang_thr, adis_timeleft;
  dReal (*avg_buf)[6];
};

struct dxJoint {
  dxWorld* world;
  dxJointGroup* group;
  int type;
  dxBody* body[2];
  int reverse;
  long long seq;             // attachment sequence number (ODE list order)
  dJointFeedback* feedback;
  void* data;                // dJointSetData
  int disabled;              // dJointDisable
  // ball / hinge / hinge2 data, FP64 as the setters compute it
  og_host::HJoint h;
  double erp, cfm;
  og::DevLimot lm1, lm2, lm3;
  double susp_erp, susp_cfm;
  // contact
  dContact contact;
};

struct dxJointGroup {
  std::vector<dxJoint*> joints;
};

struct dxHeightfieldData {
  int nx = 0, nz = 0, wrap = 0;
  double width = 0, depth = 0, scale = 1, offset = 0, thickness = 0;
  std::vector<float> heights;      // copied at build time (x fastest, then z)
  float* d_heights = nullptr;      // device copy
  bool built = false;
  // m_fMinHeight / m_fMaxHeight (heightfield.cpp:86-87, :150-237, :845-850):
  // the field's vertical extent after scale, offset and thickness, computed
  // from the samples at build time or set by dGeomHeightfieldDataSetBounds;
  // only dGeomGetAABB reads them
  float hmin = 0, hmax = 0;
};

struct dxGeom {
  int type;
  dxBody* body;
  double p[4];               // class parameters (plane normalised)
  dReal pos[4], R[12];       // own placement when not attached to a body
  dxHeightfieldData* hf;     // heightfield geoms: their data
  int placeable;             // heightfield geoms: created placeable
  int ray_flags;             // ray geoms: kRay* below
  void* data;                // dGeomSetData
  unsigned long category_bits, collide_bits;   // ~0 at creation (collision_kernel.cpp:343-368)
  int enabled;               // GEOM_ENABLED
  int zero_sized;            // GEOM_ZERO_SIZED: a zero radius or side (sphere.cpp:55 and the like)
  int has_offset;            // offset_posr != 0: placed relative to its body
  dReal opos[4], oR[12];     // the offset (body frame)
  dReal fpos[4], fR[12];     // an offset geom's own final pose, recomputed on every read
  dxGeom* body_next;         // next geom on the same body
  void* class_data;          // a user class's zeroed block (dGeomGetClassData)
  // geom transforms (collision_transform.cpp): the wrapped geom, its
  // cleanup and info modes, and its final pose as last computed
  dxGeom* tobj;
  int tcleanup, tinfo;
  dReal tpos[4], tR[12];
  const dReal *ovr_pos, *ovr_R;   // set while a transform collides or boxes this geom
  int qblock;                     // quadtree space: the block holding this geom
  int sap_dirty, sap_clean;       // sweep-and-prune space: slots in its lists (-1: none)
  // space membership (collision_kernel.h:150-171, collision_space.cpp:162-205):
  // the parent space, the intrusive list link, and the GEOM_DIRTY /
  // GEOM_AABB_BAD flags with the cached box they guard
  dxSpace* space;
  dxGeom* next;
  dxGeom** tome;
  int dirty, aabb_bad;
  dReal aabb[6];
};

// dxSpace (collision_kernel.h:190-245): a geom of a space class holding the
// list of its geoms, newest or most recently moved first
struct dxSpace : dxGeom {
  dxGeom* first;
  int count;
  int cleanup;          // destroy the geoms with the space (default 1)
  int sublevel;         // dSpaceCollide2's nesting rule
  int manual_cleanup;
  int minlevel, maxlevel;   // hash space cell levels (-3, 10)
  struct QuadTree* qt;      // quadtree space: its blocks and dirty list
  struct SapSpace* sap;     // sweep-and-prune space: its lists and sort state
};
// OPCODE's radix sort of floats as ODE 0.12 keeps it (collision_sapspace.cpp:
// 54-131, :592-820): four byte passes from the least significant, a pass
// skipped when every key has the first key's byte, negatives laid out in
// reverse in the top pass; when the keys are already in order along the
// previous result (or, with no valid result, in index order) that order is
// returned as it is. The order of equal keys follows from all of this.
struct RadixSorter {
  std::vector<uint32_t> buf;   // two rank lists
  size_t size = 0, used = 0, primary = 0;   // primary: offset of the current list
  bool valid = false;
  uint32_t* ranks1() { return buf.data() + primary; }
  uint32_t* ranks2() { return buf.data() + (primary == 0 ? size : 0); }
  void swap() { primary = primary == 0 ? size : 0; }
  const uint32_t* sort(const float* keys, uint32_t nb);
};
// dxSAPSpace (collision_sapspace.cpp:135-520): geoms in a dirty list and a
// clean list, each geom knowing its slot; removal moves the last one in
struct SapSpace {
  std::vector<dxGeom*> dirty, geoms, tmp, tmp_inf;
  std::vector<float> pos;
  RadixSorter sorter;
  int ax0, ax1, ax2;
};
// dxQuadTreeSpace (collision_quadtreespace.cpp:46-160, :334-392): a fixed tree
// of blocks split in two along x and along y per level; a geom lives in the
// smallest block whose half-open box holds its box (the root when none), in
// that block's list (newest first); geoms that moved wait in a dirty list
// and are re-seated when the space is cleaned
struct QuadBlock {
  dReal minx, maxx, miny, maxy;
  dxGeom* first;
  int count, parent, children;   // children: index of the first of four, or -1
};
struct QuadTree {
  std::vector<QuadBlock> blocks;
  std::vector<dxGeom*> dirty;
};
static bool is_space(const dxGeom* g) { return g->type >= dFirstSpaceClass && g->type <= dLastSpaceClass; }
// every attached geom is notified when its body moves (ode.cpp:362-395, util.cpp:334-336)
extern "C" {
static void body_geoms_moved(dxBody* b);
static void body_geoms_detach(dxBody* b);
static const dGeomClass* user_class_of(const dxGeom* g);
}

// dxGeom::gflags bits of a ray (ode/src/collision_kernel.h: RAY_FIRSTCONTACT,
// RAY_BACKFACECULL, RAY_CLOSEST_HIT). They steer the trimesh collider only, so
// the colliders on this path ignore them; the setters keep them for the getters.
constexpr int kRayFirstContact = 1, kRayBackfaceCull = 2, kRayClosestHit = 4;

struct dxWorld {
  double gravity[3] = {0, 0, 0};
  double erp = 0.2, cfm = 1e-5;   // dWorldCreate defaults for dSINGLE (ode/src/ode.cpp:1550-1556)
  int iterations = 20;
  double sor_w = 1.3;
  double max_vel = INFINITY, min_depth = 0;
  // body defaults of dWorldCreate (ode/src/ode.cpp:1574-1579): no damping,
  // thresholds 0.01 (kept squared), no angular speed cap
  int body_step_flags = 0;
  dReal lin_scale = 0, ang_scale = 0;
  dReal lin_thr = (dReal)0.01 * (dReal)0.01, ang_thr = (dReal)0.01 * (dReal)0.01;
  dReal max_angular_speed = INFINITY;
  // auto-disable defaults of dWorldCreate (ode/src/ode.cpp:1560-1566)
  int auto_disable = 0, adis_steps = 10;
  unsigned adis_samples = 1;
  dReal adis_time = 0;
  dReal adis_lin_thr = (dReal)0.01 * (dReal)0.01, adis_ang_thr = (dReal)0.01 * (dReal)0.01;
  std::vector<dxBody*> bodies;     // creation order
  std::vector<dxJoint*> joints;    // every live joint, creation order
  long long seq = 0;
  og::WorldCtx* ctx = nullptr;
  og::HostWorld hw;
};

namespace {

unsigned long g_seed = 0;   // ODE's global dRand state (ode/src/misc.cpp:31)
thread_local std::string g_err;

void body_sync_R(dxBody* b) {
  double q[4] = {b->q[0], b->q[1], b->q[2], b->q[3]}, R[12];
  og_host::r_from_q(R, q);
  for (int k = 0; k < 12; ++k) b->R[k] = (dReal)R[k];
}

og_host::HBody hbody(const dxBody* b) {
  og_host::HBody H;
  for (int k = 0; k < 3; ++k) H.pos[k] = b->pos[k];
  for (int k = 0; k < 4; ++k) H.q[k] = b->q[k];
  for (int k = 0; k < 12; ++k) H.R[k] = b->R[k];
  return H;
}

// The joint's two bodies as the setter helpers expect them (indices 0/1).
struct JB {
  og_host::HBody B[2];
  JB(const dxJoint* j) {
    for (int i = 0; i < 2; ++i)
      if (j->body[i]) B[i] = hbody(j->body[i]);
  }
};
void local_indices(dxJoint* j) {
  j->h.b1 = j->body[0] ? 0 : -1;
  j->h.b2 = j->body[1] ? 1 : -1;
}

void limot_default(og::DevLimot& L, const dxWorld* w) {
  // dxJointLimitMotor::init (ode/src/joints/joint.cpp:456-469)
  L.vel = 0; L.fmax = 0; L.lostop = -INFINITY; L.histop = INFINITY; L.fudge = 1;
  L.normal_cfm = (float)w->cfm; L.stop_erp = (float)w->erp; L.stop_cfm = (float)w->cfm; L.bounce = 0;
}
void limot_set(og::DevLimot& L, int num, dReal v) {
  // dxJointLimitMotor::set (ode/src/joints/joint.cpp:472-508)
  switch (num) {
    case dParamLoStop: L.lostop = v; break;
    case dParamHiStop: L.histop = v; break;
    case dParamVel: L.vel = v; break;
    case dParamFMax: if (v >= 0) L.fmax = v; break;
    case dParamFudgeFactor: if (v >= 0 && v <= 1) L.fudge = v; break;
    case dParamBounce: L.bounce = v; break;
    case dParamCFM: L.normal_cfm = v; break;
    case dParamStopERP: L.stop_erp = v; break;
    case dParamStopCFM: L.stop_cfm = v; break;
    default: break;
  }
}

dxJoint* new_joint(dxWorld* w, dxJointGroup* g, int type) {
  auto* j = new dxJoint();
  std::memset(&j->h, 0, sizeof(j->h));
  j->world = w;
  j->group = g;
  j->type = type;
  j->body[0] = j->body[1] = nullptr;
  j->h.b1 = j->h.b2 = -1;
  j->reverse = 0;
  j->seq = -1;
  j->feedback = nullptr;
  j->data = nullptr;
  j->disabled = 0;
  j->h.axis1[0] = 1;
  if (type == dJointTypeHinge2) { j->h.axis2[1] = 1; j->h.v1[0] = 1; j->h.v2[1] = 1; }
  else if (type == dJointTypeUniversal) j->h.axis2[1] = 1;
  else j->h.axis2[0] = 1;
  j->erp = w->erp;
  j->cfm = w->cfm;
  limot_default(j->lm1, w);
  limot_default(j->lm2, w);
  limot_default(j->lm3, w);
  j->susp_erp = w->erp;
  j->susp_cfm = w->cfm;
  w->joints.push_back(j);
  if (g) g->joints.push_back(j);
  return j;
}

void remove_joint(dxJoint* j) {
  auto& v = j->world->joints;
  v.erase(std::remove(v.begin(), v.end(), j), v.end());
}

// World anchor of a joint (getAnchor, ode/src/joints/joint.cpp:326-337).
void world_anchor1(const dxJoint* j, double* out) {
  const dxBody* b = j->body[0];
  double R[12], a[3];
  for (int k = 0; k < 12; ++k) R[k] = b->R[k];
  og_host::mul0_331(a, R, j->h.anchor1);
  for (int k = 0; k < 3; ++k) out[k] = a[k] + b->pos[k];
}

// getAnchor2 (ode/src/joints/joint.cpp:329-345): body 2's anchor in world
// coordinates, or the stored world point when there is no body 2
void world_anchor2(const dxJoint* j, double* out) {
  const dxBody* b = j->body[1];
  if (!b) { for (int k = 0; k < 3; ++k) out[k] = j->h.anchor2[k]; return; }
  double R[12], a[3];
  for (int k = 0; k < 12; ++k) R[k] = b->R[k];
  og_host::mul0_331(a, R, j->h.anchor2);
  for (int k = 0; k < 3; ++k) out[k] = a[k] + b->pos[k];
}
// dJointGet{Hinge,Hinge2}Anchor[2] (hinge.cpp, hinge2.cpp): the first anchor
// is body 1's unless the joint is attached reversed
void joint_anchor(const dxJoint* j, bool second, dVector3 r) {
  if (!j->body[0]) return;
  double a[3];
  if (second != (j->reverse != 0)) world_anchor2(j, a);
  else world_anchor1(j, a);
  for (int k = 0; k < 3; ++k) r[k] = (dReal)a[k];
}

}  // namespace

extern "C" {

// The collider table of collision_kernel.cpp:142-285 for what the caller can
// change in it: every class pair starts on the built-in colliders (the GPU);
// a user geom class routes its pairs that hold no collider yet to a
// first-call resolution through the class's collider getter;
// dSetColliderOverride puts the caller's function in, over what was there.
// Setting (i, j) also sets (j, i) with the geoms swapped, so for an override
// of i == j the swapped entry is the one that stays.
namespace {
constexpr int kGeomClasses = 18;                 // dGeomNumClasses of ODE 0.12
constexpr int kFirstUserClass = 14, kMaxUserClasses = 4;
enum { kColliderBuiltin = 0, kColliderUser = 1, kColliderFn = 2, kColliderTransform = 3 };
struct ColliderEntry { int kind; dColliderFn* fn; int reverse; };
ColliderEntry g_colliders[kGeomClasses][kGeomClasses];
dGeomClass g_user_classes[kMaxUserClasses];
int g_num_user_classes = 0;
void set_collider(int i, int j, int kind, dColliderFn* fn) {   // setCollider
  g_colliders[i][j] = {kind, fn, 0};
  g_colliders[j][i] = {kind, fn, 1};
}
bool is_user_class(int t) { return t >= kFirstUserClass && t < kFirstUserClass + g_num_user_classes; }
// dInitColliders (collision_kernel.cpp:167-268) for the entries that are not
// the GPU's: a geom transform pairs with every class through its own
// collider, (T, T) unswapped
bool g_colliders_ready = false;
void colliders_init() {
  if (g_colliders_ready) return;
  g_colliders_ready = true;
  const int T = dGeomTransformClass;
  for (int j = 0; j < kGeomClasses; ++j) {
    if (g_colliders[T][j].kind == kColliderBuiltin) g_colliders[T][j] = {kColliderTransform, nullptr, 0};
    if (g_colliders[j][T].kind == kColliderBuiltin) g_colliders[j][T] = {kColliderTransform, nullptr, 1};
  }
}
}  // namespace
void dSetColliderOverride(int i, int j, dColliderFn* fn) {
  if (i < 0 || j < 0 || i >= kGeomClasses || j >= kGeomClasses) return;
  colliders_init();
  set_collider(i, j, kColliderFn, fn);
}
// dCreateGeomClass (collision_kernel.cpp:975-990): at most four classes
int dCreateGeomClass(const dGeomClass* c) {
  if (!c || c->bytes < 0 || !c->collider || !c->aabb || g_num_user_classes >= kMaxUserClasses) return -1;
  colliders_init();
  g_user_classes[g_num_user_classes] = *c;
  const int cls = kFirstUserClass + g_num_user_classes;
  // setAllColliders (:162-166) through setCollider (:148-159), which writes
  // only entries that hold no collider yet
  auto empty = [](const ColliderEntry& e) { return e.kind == kColliderBuiltin || (e.kind == kColliderFn && !e.fn); };
  for (int j = 0; j < kGeomClasses; ++j) {
    if (empty(g_colliders[cls][j])) g_colliders[cls][j] = {kColliderUser, nullptr, 0};
    if (empty(g_colliders[j][cls])) g_colliders[j][cls] = {kColliderUser, nullptr, 1};
  }
  ++g_num_user_classes;
  return cls;
}
void dInitODE(void) { colliders_init(); }
int dInitODE2(unsigned int) {
  colliders_init();
  return 1;
}
// dCloseODE forgets the user classes and the caller's colliders, as the
// reference's does (odeinit.cpp:360-361)
void dCloseODE(void) {
  std::memset(g_colliders, 0, sizeof(g_colliders));
  g_num_user_classes = 0;
  g_colliders_ready = false;
}
// Per-thread data and step working memory (odeinit.cpp:515-530,
// objects.h:157-289): the GPU path keeps its own device buffers per world, so
// these accept their arguments and have nothing to do.
int dAllocateODEDataForThread(unsigned int) { return 1; }
void dCleanupODEAllDataForThread(void) {}
int dWorldUseSharedWorkingMemory(dWorldID w, dWorldID) { return w ? 1 : 0; }
void dWorldCleanupWorkingMemory(dWorldID) {}
int dWorldSetStepMemoryReservationPolicy(dWorldID w, const dWorldStepReserveInfo* info) {
  if (!w) return 0;
  return !info || (info->struct_size >= sizeof(*info) && info->reserve_factor >= 1.0f) ? 1 : 0;
}
int dWorldSetStepMemoryManager(dWorldID w, const dWorldStepMemoryFunctionsInfo* mem) {
  if (!w) return 0;
  return !mem || mem->struct_size >= sizeof(*mem) ? 1 : 0;
}
// dGetConfiguration / dCheckConfiguration (ode.cpp:2176-2275): the tokens of a
// single-precision build without debug checks or trimesh; a token matches
// whole words only, and an empty or spaced token is reported present
const char* dGetConfiguration(void) { return "ODE ODE_EXT_no_debug ODE_single_precision"; }
int dCheckConfiguration(const char* extension) {
  if (!extension || *extension == '\0' || std::strchr(extension, ' ')) return 1;
  const std::string cfg = dGetConfiguration(), tok = extension;
  for (size_t at = cfg.find(tok); at != std::string::npos; at = cfg.find(tok, at + tok.size())) {
    const size_t end = at + tok.size();
    if ((at == 0 || cfg[at - 1] == ' ') && (end == cfg.size() || cfg[end] == ' ')) return 1;
  }
  return 0;
}

// ---------------------------------------------------------------- world
dWorldID dWorldCreate(void) { return new dxWorld(); }
void dWorldDestroy(dWorldID w) {
  if (!w) return;
  for (dxJoint* j : w->joints) j->world = nullptr;
  for (dxJoint* j : std::vector<dxJoint*>(w->joints))
    if (!j->group) delete j;
  for (dxBody* b : w->bodies) {   // dBodyDestroy of each body (ode.cpp:1589-1594)
    body_geoms_detach(b);
    delete[] b->avg_buf;
    delete b;
  }
  og::ctx_destroy(w->ctx);
  delete w;
}
void dWorldSetGravity(dWorldID w, dReal x, dReal y, dReal z) { w->gravity[0] = x; w->gravity[1] = y; w->gravity[2] = z; }
void dWorldGetGravity(dWorldID w, dVector3 g) { g[0] = (dReal)w->gravity[0]; g[1] = (dReal)w->gravity[1]; g[2] = (dReal)w->gravity[2]; }
void dWorldSetERP(dWorldID w, dReal erp) { w->erp = erp; }
dReal dWorldGetERP(dWorldID w) { return (dReal)w->erp; }
void dWorldSetCFM(dWorldID w, dReal cfm) { w->cfm = cfm; }
dReal dWorldGetCFM(dWorldID w) { return (dReal)w->cfm; }
void dWorldSetQuickStepNumIterations(dWorldID w, int num) { w->iterations = num; }
int dWorldGetQuickStepNumIterations(dWorldID w) { return w->iterations; }
void dWorldSetQuickStepW(dWorldID w, dReal v) { w->sor_w = v; }
dReal dWorldGetQuickStepW(dWorldID w) { return (dReal)w->sor_w; }
void dWorldSetContactMaxCorrectingVel(dWorldID w, dReal v) { w->max_vel = v; }
dReal dWorldGetContactMaxCorrectingVel(dWorldID w) { return (dReal)w->max_vel; }
void dWorldSetContactSurfaceLayer(dWorldID w, dReal d) { w->min_depth = d; }
dReal dWorldGetContactSurfaceLayer(dWorldID w) { return (dReal)w->min_depth; }

// Damping and the angular speed cap (ode/src/ode.cpp:1038-1118, :1930-2011):
// a non-zero scale turns damping on, a finite cap turns the cap on, the
// thresholds are kept squared; bodies take the world's values at creation or
// from dBodySetDampingDefaults. dxStepBody applies them on the GPU.
dReal dWorldGetLinearDampingThreshold(dWorldID w) { return std::sqrt(w->lin_thr); }
void dWorldSetLinearDampingThreshold(dWorldID w, dReal t) { w->lin_thr = t * t; }
dReal dWorldGetAngularDampingThreshold(dWorldID w) { return std::sqrt(w->ang_thr); }
void dWorldSetAngularDampingThreshold(dWorldID w, dReal t) { w->ang_thr = t * t; }
dReal dWorldGetLinearDamping(dWorldID w) { return w->lin_scale; }
void dWorldSetLinearDamping(dWorldID w, dReal scale) {
  w->body_step_flags = scale ? (w->body_step_flags | og::kStepLinDamp) : (w->body_step_flags & ~og::kStepLinDamp);
  w->lin_scale = scale;
}
dReal dWorldGetAngularDamping(dWorldID w) { return w->ang_scale; }
void dWorldSetAngularDamping(dWorldID w, dReal scale) {
  w->body_step_flags = scale ? (w->body_step_flags | og::kStepAngDamp) : (w->body_step_flags & ~og::kStepAngDamp);
  w->ang_scale = scale;
}
void dWorldSetDamping(dWorldID w, dReal linear_scale, dReal angular_scale) {
  dWorldSetLinearDamping(w, linear_scale);
  dWorldSetAngularDamping(w, angular_scale);
}
dReal dWorldGetMaxAngularSpeed(dWorldID w) { return w->max_angular_speed; }
void dWorldSetMaxAngularSpeed(dWorldID w, dReal max_speed) {
  w->body_step_flags = max_speed < INFINITY ? (w->body_step_flags | og::kStepMaxAng)
                                            : (w->body_step_flags & ~og::kStepMaxAng);
  w->max_angular_speed = max_speed;
}
void dBodySetDampingDefaults(dBodyID b) {
  const dxWorld* w = b->world;
  b->lin_scale = w->lin_scale; b->ang_scale = w->ang_scale;
  b->lin_thr = w->lin_thr; b->ang_thr = w->ang_thr;
  const int mask = og::kStepLinDamp | og::kStepAngDamp;
  b->step_flags = (b->step_flags & ~mask) | (w->body_step_flags & mask);
}
dReal dBodyGetLinearDamping(dBodyID b) { return b->lin_scale; }
void dBodySetLinearDamping(dBodyID b, dReal scale) {
  b->step_flags = scale ? (b->step_flags | og::kStepLinDamp) : (b->step_flags & ~og::kStepLinDamp);
  b->lin_scale = scale;
}
dReal dBodyGetAngularDamping(dBodyID b) { return b->ang_scale; }
void dBodySetAngularDamping(dBodyID b, dReal scale) {
  b->step_flags = scale ? (b->step_flags | og::kStepAngDamp) : (b->step_flags & ~og::kStepAngDamp);
  b->ang_scale = scale;
}
void dBodySetDamping(dBodyID b, dReal linear_scale, dReal angular_scale) {
  dBodySetLinearDamping(b, linear_scale);
  dBodySetAngularDamping(b, angular_scale);
}
dReal dBodyGetLinearDampingThreshold(dBodyID b) { return std::sqrt(b->lin_thr); }
void dBodySetLinearDampingThreshold(dBodyID b, dReal t) { b->lin_thr = t * t; }
dReal dBodyGetAngularDampingThreshold(dBodyID b) { return std::sqrt(b->ang_thr); }
void dBodySetAngularDampingThreshold(dBodyID b, dReal t) { b->ang_thr = t * t; }
dReal dBodyGetMaxAngularSpeed(dBodyID b) { return b->max_angular_speed; }
void dBodySetMaxAngularSpeed(dBodyID b, dReal max_speed) {
  b->step_flags = max_speed < INFINITY ? (b->step_flags | og::kStepMaxAng) : (b->step_flags & ~og::kStepMaxAng);
  b->max_angular_speed = max_speed;
}
// Finite rotation (ode/src/ode.cpp:767-806): the mode, and an axis that, when
// non-zero, is normalised and limits the finite part to rotation about it
void dBodySetFiniteRotationMode(dBodyID b, int mode) {
  b->step_flags &= ~(og::kStepFiniteRot | og::kStepFiniteAxis);
  if (mode) {
    b->step_flags |= og::kStepFiniteRot;
    if (b->frot_axis[0] != 0 || b->frot_axis[1] != 0 || b->frot_axis[2] != 0) b->step_flags |= og::kStepFiniteAxis;
  }
}
void dBodySetFiniteRotationAxis(dBodyID b, dReal x, dReal y, dReal z) {
  b->frot_axis[0] = x; b->frot_axis[1] = y; b->frot_axis[2] = z;
  if (x != 0 || y != 0 || z != 0) {
    dNormalize3(b->frot_axis);
    b->step_flags |= og::kStepFiniteAxis;
  } else {
    b->step_flags &= ~og::kStepFiniteAxis;
  }
}
int dBodyGetFiniteRotationMode(dBodyID b) { return (b->step_flags & og::kStepFiniteRot) != 0; }
void dBodyGetFiniteRotationAxis(dBodyID b, dVector3 result) {
  for (int k = 0; k < 3; ++k) result[k] = b->frot_axis[k];
}
// Called after each step for every body, in island order, once all bodies
// have their new state (ODE calls it as each body is stepped).
// Auto-disable parameters (ode/src/ode.cpp:900-1010, :1843-1927): thresholds
// kept squared; a body takes the world's at creation or from
// dBodySetAutoDisableDefaults; turning a body's flag off also enables it and
// resets its countdowns and samples to the world's.
dReal dWorldGetAutoDisableLinearThreshold(dWorldID w) { return std::sqrt(w->adis_lin_thr); }
void dWorldSetAutoDisableLinearThreshold(dWorldID w, dReal t) { w->adis_lin_thr = t * t; }
dReal dWorldGetAutoDisableAngularThreshold(dWorldID w) { return std::sqrt(w->adis_ang_thr); }
void dWorldSetAutoDisableAngularThreshold(dWorldID w, dReal t) { w->adis_ang_thr = t * t; }
int dWorldGetAutoDisableAverageSamplesCount(dWorldID w) { return (int)w->adis_samples; }
void dWorldSetAutoDisableAverageSamplesCount(dWorldID w, unsigned int n) { w->adis_samples = n; }
int dWorldGetAutoDisableSteps(dWorldID w) { return w->adis_steps; }
void dWorldSetAutoDisableSteps(dWorldID w, int steps) { w->adis_steps = steps; }
dReal dWorldGetAutoDisableTime(dWorldID w) { return w->adis_time; }
void dWorldSetAutoDisableTime(dWorldID w, dReal time) { w->adis_time = time; }
// the raw flag bit, as ODE 0.12 returns it (ode.cpp:1913-1917)
int dWorldGetAutoDisableFlag(dWorldID w) { return w->auto_disable ? 16 : 0; }
void dWorldSetAutoDisableFlag(dWorldID w, int do_auto_disable) { w->auto_disable = do_auto_disable != 0; }
dReal dBodyGetAutoDisableLinearThreshold(dBodyID b) { return std::sqrt(b->adis_lin_thr); }
void dBodySetAutoDisableLinearThreshold(dBodyID b, dReal t) { b->adis_lin_thr = t * t; }
dReal dBodyGetAutoDisableAngularThreshold(dBodyID b) { return std::sqrt(b->adis_ang_thr); }
void dBodySetAutoDisableAngularThreshold(dBodyID b, dReal t) { b->adis_ang_thr = t * t; }
int dBodyGetAutoDisableAverageSamplesCount(dBodyID b) { return (int)b->adis_samples; }
void dBodySetAutoDisableAverageSamplesCount(dBodyID b, unsigned int n) {
  b->adis_samples = n;
  delete[] b->avg_buf;
  b->avg_buf = n > 0 ? new dReal[n][6] : nullptr;
  b->avg_counter = 0;
  b->avg_ready = 0;
}
int dBodyGetAutoDisableSteps(dBodyID b) { return b->adis_steps; }
void dBodySetAutoDisableSteps(dBodyID b, int steps) { b->adis_steps = steps; }
dReal dBodyGetAutoDisableTime(dBodyID b) { return b->adis_time; }
void dBodySetAutoDisableTime(dBodyID b, dReal time) { b->adis_time = time; }
int dBodyGetAutoDisableFlag(dBodyID b) { return b->auto_disable ? 1 : 0; }
void dBodySetAutoDisableFlag(dBodyID b, int do_auto_disable) {
  if (!do_auto_disable) {
    b->auto_disable = 0;
    b->disabled = 0;
    b->adis_steps = b->world->adis_steps;
    b->adis_time = b->world->adis_time;
    dBodySetAutoDisableAverageSamplesCount(b, b->world->adis_samples);
  } else {
    b->auto_disable = 1;
  }
}
void dBodySetAutoDisableDefaults(dBodyID b) {
  const dxWorld* w = b->world;
  b->adis_steps = w->adis_steps; b->adis_time = w->adis_time; b->adis_samples = w->adis_samples;
  b->adis_lin_thr = w->adis_lin_thr; b->adis_ang_thr = w->adis_ang_thr;
  dBodySetAutoDisableFlag(b, w->auto_disable);
}
void dBodySetMovedCallback(dBodyID b, void (*callback)(dBodyID)) { b->moved_callback = callback; }
// dBodyEnable / Disable / IsEnabled (ode.cpp:854-875); a body also changes
// state when a step's auto-disable check or island walk reaches it
void dBodyEnable(dBodyID b) {
  b->disabled = 0;
  b->adis_stepsleft = b->adis_steps;
  b->adis_timeleft = b->adis_time;
}
void dBodyDisable(dBodyID b) { b->disabled = 1; }
int dBodyIsEnabled(dBodyID b) { return b->disabled ? 0 : 1; }
dGeomID dBodyGetFirstGeom(dBodyID b) { return b->geom; }        // ode.cpp:1122-1133
dGeomID dBodyGetNextGeom(dGeomID g) { return g->body_next; }

// ---------------------------------------------------------------- bodies
dBodyID dBodyCreate(dWorldID w) {
  // dBodyCreate defaults (ode/src/ode.cpp:248-294): unit mass and inertia,
  // identity orientation, gyroscopic flag on
  auto* b = new dxBody();
  std::memset(b, 0, sizeof(*b));
  b->world = w;
  b->q[0] = 1;
  body_sync_R(b);
  dMassSetParameters(&b->mass, 1, 0, 0, 0, 1, 1, 1, 0, 0, 0);
  for (int k = 0; k < 9; ++k) b->invI[k] = (k % 4 == 0) ? 1.0 : 0.0;
  b->invMass = 1;
  b->flags = ODEGPU_BODY_GYROSCOPIC;
  w->bodies.push_back(b);
  // auto-disable state (ode.cpp:270-279)
  dBodySetAutoDisableDefaults(b);
  b->adis_stepsleft = b->adis_steps;
  b->adis_timeleft = b->adis_time;
  dBodySetAutoDisableAverageSamplesCount(b, b->adis_samples);
  dBodySetDampingDefaults(b);   // ode.cpp:285-288
  b->step_flags |= w->body_step_flags & og::kStepMaxAng;
  b->max_angular_speed = w->max_angular_speed;
  return b;
}
void dBodyDestroy(dBodyID b) {
  if (!b) return;
  body_geoms_detach(b);
  dxWorld* w = b->world;
  for (dxJoint* j : w->joints) {
    for (int i = 0; i < 2; ++i)
      if (j->body[i] == b) j->body[i] = nullptr;
    if (!j->body[0] && j->body[1]) { j->body[0] = j->body[1]; j->body[1] = nullptr; j->reverse = 1; }
  }
  w->bodies.erase(std::remove(w->bodies.begin(), w->bodies.end(), b), w->bodies.end());
  delete[] b->avg_buf;
  delete b;
}
void dBodySetPosition(dBodyID b, dReal x, dReal y, dReal z) {
  b->pos[0] = x; b->pos[1] = y; b->pos[2] = z;
  body_geoms_moved(b);
}
void dBodySetQuaternion(dBodyID b, const dQuaternion q) {
  double qd[4] = {q[0], q[1], q[2], q[3]};
  og_host::normalize4(qd);
  for (int k = 0; k < 4; ++k) b->q[k] = (dReal)qd[k];
  body_sync_R(b);
  body_geoms_moved(b);
}
void dBodySetRotation(dBodyID b, const dMatrix3 R) {
  // dQfromR (ode/src/rotation.cpp:258-307), then normalise as dBodySetRotation does
  double r[12], q[4];
  for (int k = 0; k < 12; ++k) r[k] = R[k];
  auto Rr = [&](int i, int j) { return r[i * 4 + j]; };
  double tr = Rr(0, 0) + Rr(1, 1) + Rr(2, 2);
  if (tr >= 0) {
    double s = std::sqrt(tr + 1);
    q[0] = 0.5 * s; s = 0.5 / s;
    q[1] = (Rr(2, 1) - Rr(1, 2)) * s; q[2] = (Rr(0, 2) - Rr(2, 0)) * s; q[3] = (Rr(1, 0) - Rr(0, 1)) * s;
  } else {
    int c = (Rr(1, 1) > Rr(0, 0)) ? ((Rr(2, 2) > Rr(1, 1)) ? 2 : 1) : ((Rr(2, 2) > Rr(0, 0)) ? 2 : 0);
    if (c == 0) {
      double s = std::sqrt((Rr(0, 0) - (Rr(1, 1) + Rr(2, 2))) + 1);
      q[1] = 0.5 * s; s = 0.5 / s;
      q[2] = (Rr(0, 1) + Rr(1, 0)) * s; q[3] = (Rr(2, 0) + Rr(0, 2)) * s; q[0] = (Rr(2, 1) - Rr(1, 2)) * s;
    } else if (c == 1) {
      double s = std::sqrt((Rr(1, 1) - (Rr(2, 2) + Rr(0, 0))) + 1);
      q[2] = 0.5 * s; s = 0.5 / s;
      q[3] = (Rr(1, 2) + Rr(2, 1)) * s; q[1] = (Rr(0, 1) + Rr(1, 0)) * s; q[0] = (Rr(0, 2) - Rr(2, 0)) * s;
    } else {
      double s = std::sqrt((Rr(2, 2) - (Rr(0, 0) + Rr(1, 1))) + 1);
      q[3] = 0.5 * s; s = 0.5 / s;
      q[1] = (Rr(2, 0) + Rr(0, 2)) * s; q[2] = (Rr(1, 2) + Rr(2, 1)) * s; q[0] = (Rr(1, 0) - Rr(0, 1)) * s;
    }
  }
  og_host::normalize4(q);
  for (int k = 0; k < 4; ++k) b->q[k] = (dReal)q[k];
  body_sync_R(b);
  body_geoms_moved(b);
}
void dBodySetLinearVel(dBodyID b, dReal x, dReal y, dReal z) { b->lvel[0] = x; b->lvel[1] = y; b->lvel[2] = z; }
void dBodySetAngularVel(dBodyID b, dReal x, dReal y, dReal z) { b->avel[0] = x; b->avel[1] = y; b->avel[2] = z; }
const dReal* dBodyGetPosition(dBodyID b) { return b->pos; }
const dReal* dBodyGetRotation(dBodyID b) { return b->R; }
const dReal* dBodyGetQuaternion(dBodyID b) { return b->q; }
const dReal* dBodyGetLinearVel(dBodyID b) { return b->lvel; }
const dReal* dBodyGetAngularVel(dBodyID b) { return b->avel; }
// Kinematic bodies (ode/src/ode.cpp:834-852): zero inverse mass and inertia,
// so forces and constraints do not move them; dBodySetDynamic restores both
// from the body's mass.
void dBodySetKinematic(dBodyID b) {
  for (int k = 0; k < 9; ++k) b->invI[k] = 0;
  b->invMass = 0;
}
int dBodyIsKinematic(dBodyID b) { return b->invMass == 0; }
void dBodySetDynamic(dBodyID b) {
  const dMass m = b->mass;
  dBodySetMass(b, &m);
}
void dBodySetMass(dBodyID b, const dMass* m) {
  // dBodySetMass (ode/src/ode.cpp:492-509): invI through a Cholesky inverse
  b->mass = *m;
  double I[9], inv[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) I[r * 3 + c] = m->I[r * 4 + c];
  if (!og_host::invert_pd3(I, inv))
    for (int k = 0; k < 9; ++k) inv[k] = (k % 4 == 0) ? 1.0 : 0.0;
  for (int k = 0; k < 9; ++k) b->invI[k] = inv[k];
  b->invMass = 1.0 / m->mass;
}
void dBodyGetMass(dBodyID b, dMass* m) { *m = b->mass; }
void dBodyAddForce(dBodyID b, dReal x, dReal y, dReal z) { b->facc[0] += x; b->facc[1] += y; b->facc[2] += z; }
void dBodyAddTorque(dBodyID b, dReal x, dReal y, dReal z) { b->tacc[0] += x; b->tacc[1] += y; b->tacc[2] += z; }
const dReal* dBodyGetForce(dBodyID b) { return b->facc; }
const dReal* dBodyGetTorque(dBodyID b) { return b->tacc; }
void dBodySetGravityMode(dBodyID b, int mode) {
  if (mode) b->flags &= ~ODEGPU_BODY_NO_GRAVITY; else b->flags |= ODEGPU_BODY_NO_GRAVITY;
}
int dBodyGetGravityMode(dBodyID b) { return (b->flags & ODEGPU_BODY_NO_GRAVITY) == 0; }
void dBodySetGyroscopicMode(dBodyID b, int e) {
  if (e) b->flags |= ODEGPU_BODY_GYROSCOPIC; else b->flags &= ~ODEGPU_BODY_GYROSCOPIC;
}
int dBodyGetGyroscopicMode(dBodyID b) { return (b->flags & ODEGPU_BODY_GYROSCOPIC) != 0; }

// ---------------------------------------------------------------- mass
void dMassSetZero(dMass* m) { std::memset(m, 0, sizeof(*m)); }
void dMassSetParameters(dMass* m, dReal themass, dReal cgx, dReal cgy, dReal cgz, dReal I11, dReal I22,
                        dReal I33, dReal I12, dReal I13, dReal I23) {
  // ode/src/mass.cpp:94-117
  dMassSetZero(m);
  m->mass = themass;
  m->c[0] = cgx; m->c[1] = cgy; m->c[2] = cgz;
  m->I[0] = I11; m->I[5] = I22; m->I[10] = I33;
  m->I[1] = I12; m->I[2] = I13; m->I[6] = I23;
  m->I[4] = I12; m->I[8] = I13; m->I[9] = I23;
}
void dMassSetSphereTotal(dMass* m, dReal total, dReal r) {
  const dReal ii = 0.4f * total * r * r;  // ode/src/mass.cpp:126-137
  dMassSetParameters(m, total, 0, 0, 0, ii, ii, ii, 0, 0, 0);
}
void dMassSetSphere(dMass* m, dReal density, dReal r) {
  dMassSetSphereTotal(m, (dReal)((4.0 / 3.0) * M_PI * r * r * r * density), r);
}
void dMassSetBoxTotal(dMass* m, dReal total, dReal lx, dReal ly, dReal lz) {
  // ode/src/mass.cpp:208-222
  dMassSetParameters(m, total, 0, 0, 0, total / 12.0f * (ly * ly + lz * lz), total / 12.0f * (lx * lx + lz * lz),
                     total / 12.0f * (lx * lx + ly * ly), 0, 0, 0);
}
void dMassSetBox(dMass* m, dReal density, dReal lx, dReal ly, dReal lz) {
  dMassSetBoxTotal(m, lx * ly * lz * density, lx, ly, lz);
}
void dMassAdjust(dMass* m, dReal newmass) {
  // ode/src/mass.cpp:441-451
  const dReal scale = newmass / m->mass;
  m->mass = newmass;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) m->I[i * 4 + j] *= scale;
}
void dMassSetCapsule(dMass* m, dReal density, int direction, dReal radius, dReal length) {
  // ode/src/mass.cpp:140-165: cylinder part plus the two hemispherical caps
  if (direction < 1 || direction > 3) return;
  dMassSetZero(m);
  const dReal M1 = (dReal)(M_PI * radius * radius * length * density);
  const dReal M2 = (dReal)((4.0f / 3.0f) * M_PI * radius * radius * radius * density);
  m->mass = M1 + M2;
  const dReal Ia = M1 * (0.25f * radius * radius + (1.0f / 12.0f) * length * length) +
                   M2 * (0.4f * radius * radius + 0.375f * radius * length + 0.25f * length * length);
  const dReal Ib = (M1 * 0.5f + M2 * 0.4f) * radius * radius;
  m->I[0] = m->I[5] = m->I[10] = Ia;
  m->I[(direction - 1) * 5] = Ib;
}
void dMassSetCapsuleTotal(dMass* m, dReal total_mass, int direction, dReal radius, dReal length) {
  dMassSetCapsule(m, 1.0f, direction, radius, length);
  dMassAdjust(m, total_mass);
}
void dMassSetCylinderTotal(dMass* m, dReal total_mass, int direction, dReal radius, dReal length) {
  // ode/src/mass.cpp:180-200
  if (direction < 1 || direction > 3) return;
  dMassSetZero(m);
  const dReal r2 = radius * radius;
  m->mass = total_mass;
  const dReal I = total_mass * (0.25f * r2 + (1.0f / 12.0f) * length * length);
  m->I[0] = m->I[5] = m->I[10] = I;
  m->I[(direction - 1) * 5] = total_mass * 0.5f * r2;
}
void dMassSetCylinder(dMass* m, dReal density, int direction, dReal radius, dReal length) {
  dMassSetCylinderTotal(m, (dReal)(M_PI * radius * radius * length * density), direction, radius, length);
}

// ---------------------------------------------------------------- joints
dJointID dJointCreateBall(dWorldID w, dJointGroupID g) { return new_joint(w, g, dJointTypeBall); }
dJointID dJointCreateHinge(dWorldID w, dJointGroupID g) { return new_joint(w, g, dJointTypeHinge); }
dJointID dJointCreateHinge2(dWorldID w, dJointGroupID g) { return new_joint(w, g, dJointTypeHinge2); }
dJointID dJointCreateSlider(dWorldID w, dJointGroupID g) { return new_joint(w, g, dJointTypeSlider); }
dJointID dJointCreateUniversal(dWorldID w, dJointGroupID g) { return new_joint(w, g, dJointTypeUniversal); }
dJointID dJointCreateFixed(dWorldID w, dJointGroupID g) { return new_joint(w, g, dJointTypeFixed); }
dJointID dJointCreateAMotor(dWorldID w, dJointGroupID g) { return new_joint(w, g, dJointTypeAMotor); }
// dJointCreateNull (ode.cpp:1250-1254, joints/null.cpp): no rows, but it joins
// its bodies into one island like any joint
dJointID dJointCreateNull(dWorldID w, dJointGroupID g) { return new_joint(w, g, dJointTypeNull); }
dJointID dJointCreateContact(dWorldID w, dJointGroupID g, const dContact* c) {
  dxJoint* j = new_joint(w, g, dJointTypeContact);
  j->contact = *c;   // dJointCreateContact copies the contact (ode/src/ode.cpp:1201-1208)
  return j;
}
void dJointDestroy(dJointID j) {
  if (!j || j->group) return;   // group joints go with their group (ode/src/ode.cpp:1248)
  if (j->world) remove_joint(j);
  delete j;
}
dJointGroupID dJointGroupCreate(int) { return new dxJointGroup(); }
void dJointGroupEmpty(dJointGroupID g) {
  if (!g) return;
  for (dxJoint* j : g->joints) {
    if (j->world) remove_joint(j);
    delete j;
  }
  g->joints.clear();
}
void dJointGroupDestroy(dJointGroupID g) {
  dJointGroupEmpty(g);
  delete g;
}
void dJointAttach(dJointID j, dBodyID b1, dBodyID b2) {
  // ode/src/ode.cpp:1348-1399: a missing body1 moves to body2's slot
  if (!b1) { b1 = b2; b2 = nullptr; j->reverse = 1; } else j->reverse = 0;
  j->body[0] = b1;
  j->body[1] = b2;
  j->seq = j->world->seq++;
  local_indices(j);
  if (!b1) return;
  // setRelativeValues (ball.cpp:175-180, hinge.cpp:364-373, hinge2.cpp:425-448)
  JB jb(j);
  og_host::HJoint& H = j->h;
  if (j->type == dJointTypeBall || j->type == dJointTypeHinge) {
    double a[3];
    if (j->reverse) { for (int k = 0; k < 3; ++k) a[k] = H.anchor2[k]; }
    else world_anchor1(j, a);
    og_host::set_anchors(H, jb.B, a[0], a[1], a[2], H.anchor1, H.anchor2);
    if (j->type == dJointTypeHinge) {
      double ax[3];
      og_host::mul0_331(ax, jb.B[0].R, H.axis1);
      og_host::set_axes(H, jb.B, ax[0], ax[1], ax[2], H.axis1, H.axis2);
      og_host::hinge_qrel(H, jb.B);
    }
  } else if (j->type == dJointTypeSlider) {
    // slider.cpp:349-353
    og_host::slider_offset(H, jb.B);
    og_host::initial_qrel(H, jb.B);
  } else if (j->type == dJointTypeUniversal) {
    // universal.cpp:772-796: anchor and axes re-expressed in the new bodies'
    // frames (a reversed joint's anchor getter has no body 2 and leaves the
    // anchor alone here)
    double a[3], ax1[3], ax2[3];
    if (j->reverse) { for (int k = 0; k < 3; ++k) a[k] = H.anchor2[k]; }
    else world_anchor1(j, a);
    og_host::set_anchors(H, jb.B, a[0], a[1], a[2], H.anchor1, H.anchor2);
    og_host::universal_axes(H, jb.B, ax1, ax2);
    if (j->reverse) {
      og_host::set_axes(H, jb.B, ax2[0], ax2[1], ax2[2], nullptr, H.axis2);
      og_host::set_axes(H, jb.B, ax1[0], ax1[1], ax1[2], H.axis1, nullptr);
    } else {
      og_host::set_axes(H, jb.B, ax1[0], ax1[1], ax1[2], H.axis1, nullptr);
      og_host::set_axes(H, jb.B, ax2[0], ax2[1], ax2[2], nullptr, H.axis2);
    }
    og_host::universal_qrels(H, jb.B);
  } else if (j->type == dJointTypeHinge2 && b2) {
    double a[3], ax[3];
    world_anchor1(j, a);
    og_host::set_anchors(H, jb.B, a[0], a[1], a[2], H.anchor1, H.anchor2);
    og_host::mul0_331(ax, jb.B[0].R, H.axis1);
    og_host::set_axes(H, jb.B, ax[0], ax[1], ax[2], H.axis1, nullptr);
    og_host::mul0_331(ax, jb.B[1].R, H.axis2);
    og_host::set_axes(H, jb.B, ax[0], ax[1], ax[2], nullptr, H.axis2);
    og_host::hinge2_axis_info(H, jb.B);
    og_host::hinge2_make_v(H, jb.B);
  }
}
dJointType dJointGetType(dJointID j) { return (dJointType)j->type; }
dBodyID dJointGetBody(dJointID j, int index) {
  // ode/src/ode.cpp:1415-1436 (reverse flag swaps the reported order)
  if (index == 0 || index == 1) {
    if (j->reverse) return j->body[1 - index];
    return j->body[index];
  }
  return nullptr;
}
void dJointSetFeedback(dJointID j, dJointFeedback* f) { j->feedback = f; }
dJointFeedback* dJointGetFeedback(dJointID j) { return j->feedback; }

void dJointSetBallAnchor(dJointID j, dReal x, dReal y, dReal z) {
  JB jb(j);
  og_host::set_anchors(j->h, jb.B, x, y, z, j->h.anchor1, j->h.anchor2);
}
void dJointSetBallParam(dJointID j, int p, dReal v) {
  if (p == dParamCFM) j->cfm = v; else if (p == dParamERP) j->erp = v;
}
void dJointGetBallAnchor(dJointID j, dVector3 r) {
  double a[3];
  if (j->body[0]) { world_anchor1(j, a); for (int k = 0; k < 3; ++k) r[k] = (dReal)a[k]; }
}
void dJointSetHingeAnchor(dJointID j, dReal x, dReal y, dReal z) {
  JB jb(j);
  og_host::set_anchors(j->h, jb.B, x, y, z, j->h.anchor1, j->h.anchor2);
  og_host::hinge_qrel(j->h, jb.B);
}
void dJointGetHingeAnchor(dJointID j, dVector3 r) { joint_anchor(j, false, r); }
void dJointGetHingeAnchor2(dJointID j, dVector3 r) { joint_anchor(j, true, r); }
void dJointGetHinge2Anchor(dJointID j, dVector3 r) { joint_anchor(j, false, r); }
void dJointGetHinge2Anchor2(dJointID j, dVector3 r) { joint_anchor(j, true, r); }
void dJointSetHingeAxis(dJointID j, dReal x, dReal y, dReal z) {
  JB jb(j);
  og_host::set_axes(j->h, jb.B, x, y, z, j->h.axis1, j->h.axis2);
  og_host::hinge_qrel(j->h, jb.B);
}
void dJointSetHingeParam(dJointID j, int p, dReal v) { limot_set(j->lm1, p, v); }
dReal dJointGetHingeAngle(dJointID j) {
  // getHingeAngle (ode/src/joints/joint.cpp:381-451), FP64 on the host
  if (!j->body[0]) return 0;
  double q1[4], qrel[4], qq[4];
  for (int k = 0; k < 4; ++k) q1[k] = j->body[0]->q[k];
  if (j->body[1]) {
    double q2[4];
    for (int k = 0; k < 4; ++k) q2[k] = j->body[1]->q[k];
    og_host::qmul1(qq, q1, q2);
    // qrel = qq * conj(qrel0) (dQMultiply2)
    const double* c = j->h.qrel;
    qrel[0] = qq[0] * c[0] + qq[1] * c[1] + qq[2] * c[2] + qq[3] * c[3];
    qrel[1] = -qq[0] * c[1] + qq[1] * c[0] - qq[2] * c[3] + qq[3] * c[2];
    qrel[2] = -qq[0] * c[2] + qq[2] * c[0] - qq[3] * c[1] + qq[1] * c[3];
    qrel[3] = -qq[0] * c[3] + qq[3] * c[0] - qq[1] * c[2] + qq[2] * c[1];
  } else {
    const double* c = j->h.qrel;   // dQMultiply3
    qrel[0] = q1[0] * c[0] - q1[1] * c[1] - q1[2] * c[2] - q1[3] * c[3];
    qrel[1] = -q1[0] * c[1] - q1[1] * c[0] + q1[2] * c[3] - q1[3] * c[2];
    qrel[2] = -q1[0] * c[2] - q1[2] * c[0] + q1[3] * c[1] - q1[1] * c[3];
    qrel[3] = -q1[0] * c[3] - q1[3] * c[0] + q1[1] * c[2] - q1[2] * c[1];
  }
  const double cost2 = qrel[0];
  const double sint2 = std::sqrt(qrel[1] * qrel[1] + qrel[2] * qrel[2] + qrel[3] * qrel[3]);
  double theta = (og_host::dot3(qrel + 1, j->h.axis1) >= 0) ? 2 * std::atan2(sint2, cost2)
                                                             : 2 * std::atan2(sint2, -cost2);
  if (theta > M_PI) theta -= 2 * M_PI;
  theta = -theta;
  return (dReal)(j->reverse ? -theta : theta);
}
dReal dJointGetHingeAngleRate(dJointID j) {
  if (!j->body[0]) return 0;
  double R[12], ax[3];
  for (int k = 0; k < 12; ++k) R[k] = j->body[0]->R[k];
  og_host::mul0_331(ax, R, j->h.axis1);
  double rate = ax[0] * j->body[0]->avel[0] + ax[1] * j->body[0]->avel[1] + ax[2] * j->body[0]->avel[2];
  if (j->body[1]) rate -= ax[0] * j->body[1]->avel[0] + ax[1] * j->body[1]->avel[1] + ax[2] * j->body[1]->avel[2];
  return (dReal)(j->reverse ? -rate : rate);
}
void dJointAddHingeTorque(dJointID j, dReal torque) {
  // ode/src/joints/hinge.cpp:326-345
  if (j->reverse) torque = -torque;
  if (!j->body[0]) return;
  dReal ax[3];
  for (int r = 0; r < 3; ++r)
    ax[r] = (dReal)(j->body[0]->R[r * 4] * j->h.axis1[0] + j->body[0]->R[r * 4 + 1] * j->h.axis1[1] +
                    j->body[0]->R[r * 4 + 2] * j->h.axis1[2]) * torque;
  dBodyAddTorque(j->body[0], ax[0], ax[1], ax[2]);
  if (j->body[1]) dBodyAddTorque(j->body[1], -ax[0], -ax[1], -ax[2]);
}
void dJointSetHinge2Anchor(dJointID j, dReal x, dReal y, dReal z) {
  JB jb(j);
  og_host::set_anchors(j->h, jb.B, x, y, z, j->h.anchor1, j->h.anchor2);
  og_host::hinge2_make_v(j->h, jb.B);
}
void dJointSetHinge2Axis1(dJointID j, dReal x, dReal y, dReal z) {
  JB jb(j);
  if (j->body[0]) {
    og_host::set_axes(j->h, jb.B, x, y, z, j->h.axis1, nullptr);
    if (j->body[1]) og_host::hinge2_axis_info(j->h, jb.B);
  }
  og_host::hinge2_make_v(j->h, jb.B);
}
void dJointSetHinge2Axis2(dJointID j, dReal x, dReal y, dReal z) {
  JB jb(j);
  if (j->body[1]) {
    og_host::set_axes(j->h, jb.B, x, y, z, nullptr, j->h.axis2);
    og_host::hinge2_axis_info(j->h, jb.B);
  }
  og_host::hinge2_make_v(j->h, jb.B);
}
void dJointSetHinge2Param(dJointID j, int p, dReal v) {
  // ode/src/joints/hinge2.cpp:259-274
  if ((p & 0xff00) == 0x100) limot_set(j->lm2, p & 0xff, v);
  else if (p == dParamSuspensionERP) j->susp_erp = v;
  else if (p == dParamSuspensionCFM) j->susp_cfm = v;
  else limot_set(j->lm1, p, v);
}
void dJointAddHinge2Torques(dJointID j, dReal t1, dReal t2) {
  // ode/src/joints/hinge2.cpp:393-410
  if (!j->body[0] || !j->body[1]) return;
  dReal a1[3], a2[3];
  for (int r = 0; r < 3; ++r) {
    a1[r] = (dReal)(j->body[0]->R[r * 4] * j->h.axis1[0] + j->body[0]->R[r * 4 + 1] * j->h.axis1[1] +
                    j->body[0]->R[r * 4 + 2] * j->h.axis1[2]);
    a2[r] = (dReal)(j->body[1]->R[r * 4] * j->h.axis2[0] + j->body[1]->R[r * 4 + 1] * j->h.axis2[1] +
                    j->body[1]->R[r * 4 + 2] * j->h.axis2[2]);
  }
  dReal t[3] = {a1[0] * t1 + a2[0] * t2, a1[1] * t1 + a2[1] * t2, a1[2] * t1 + a2[2] * t2};
  dBodyAddTorque(j->body[0], t[0], t[1], t[2]);
  dBodyAddTorque(j->body[1], -t[0], -t[1], -t[2]);
}
dReal dJointGetHinge2Angle1(dJointID j) {
  // dxJointHinge2::measureAngle (ode/src/joints/hinge2.cpp:33-41)
  if (!j->body[0] || !j->body[1]) return 0;
  double R1[12], R2[12], a1[3], a2[3];
  for (int k = 0; k < 12; ++k) { R1[k] = j->body[0]->R[k]; R2[k] = j->body[1]->R[k]; }
  og_host::mul0_331(a1, R2, j->h.axis2);
  og_host::mul1_331(a2, R1, a1);
  return (dReal)(-std::atan2(og_host::dot3(j->h.v2, a2), og_host::dot3(j->h.v1, a2)));
}
dReal limot_get(const og::DevLimot& L, int num) {
  // dxJointLimitMotor::get (ode/src/joints/joint.cpp:506-532)
  switch (num) {
    case dParamLoStop: return L.lostop;
    case dParamHiStop: return L.histop;
    case dParamVel: return L.vel;
    case dParamFMax: return L.fmax;
    case dParamFudgeFactor: return L.fudge;
    case dParamBounce: return L.bounce;
    case dParamCFM: return L.normal_cfm;
    case dParamStopERP: return L.stop_erp;
    case dParamStopCFM: return L.stop_cfm;
    default: return 0;
  }
}
// World-frame axis of body 1 / body 2 (getAxis / getAxis2, ode/src/joints/joint.cpp:357-378).
void world_axis1(const dxJoint* j, const double* axis, dVector3 r) {
  if (!j->body[0]) return;
  double R[12], a[3];
  for (int k = 0; k < 12; ++k) R[k] = j->body[0]->R[k];
  og_host::mul0_331(a, R, axis);
  for (int k = 0; k < 3; ++k) r[k] = (dReal)a[k];
}
void world_axis2(const dxJoint* j, const double* axis, dVector3 r) {
  if (j->body[1]) {
    double R[12], a[3];
    for (int k = 0; k < 12; ++k) R[k] = j->body[1]->R[k];
    og_host::mul0_331(a, R, axis);
    for (int k = 0; k < 3; ++k) r[k] = (dReal)a[k];
  } else {
    for (int k = 0; k < 3; ++k) r[k] = (dReal)axis[k];
  }
}

// hinge / hinge2 axes in world coordinates (hinge.cpp, hinge2.cpp)
void dJointGetHingeAxis(dJointID j, dVector3 r) { world_axis1(j, j->h.axis1, r); }
void dJointGetHinge2Axis1(dJointID j, dVector3 r) { world_axis1(j, j->h.axis1, r); }
void dJointGetHinge2Axis2(dJointID j, dVector3 r) {
  if (j->body[1]) world_axis2(j, j->h.axis2, r);
}

// slider (ode/src/joints/slider.cpp)
void dJointSetSliderAxis(dJointID j, dReal x, dReal y, dReal z) {
  // :250-258
  JB jb(j);
  og_host::set_axes(j->h, jb.B, x, y, z, j->h.axis1, nullptr);
  og_host::slider_offset(j->h, jb.B);
  og_host::initial_qrel(j->h, jb.B);
}
void dJointGetSliderAxis(dJointID j, dVector3 r) { world_axis1(j, j->h.axis1, r); }
void dJointSetSliderParam(dJointID j, int p, dReal v) { limot_set(j->lm1, p, v); }
dReal dJointGetSliderParam(dJointID j, int p) { return limot_get(j->lm1, p); }
dReal dJointGetSliderPosition(dJointID j) {
  if (!j->body[0]) return 0;
  JB jb(j);
  return (dReal)og_host::slider_position(j->h, jb.B);
}
dReal dJointGetSliderPositionRate(dJointID j) {
  // :82-104
  if (!j->body[0]) return 0;
  dVector3 ax;
  world_axis1(j, j->h.axis1, ax);
  const dReal* v1 = j->body[0]->lvel;
  if (j->body[1]) {
    const dReal* v2 = j->body[1]->lvel;
    return ax[0] * v1[0] + ax[1] * v1[1] + ax[2] * v1[2] - (ax[0] * v2[0] + ax[1] * v2[1] + ax[2] * v2[2]);
  }
  dReal rate = ax[0] * v1[0] + ax[1] * v1[1] + ax[2] * v1[2];
  return j->reverse ? -rate : rate;
}
void dJointAddSliderForce(dJointID j, dReal force) {
  // :305-342; on a reversed joint the reference computes force -= force (zero)
  if (j->reverse) force -= force;
  dVector3 ax = {0, 0, 0, 0};
  world_axis1(j, j->h.axis1, ax);
  for (int k = 0; k < 3; ++k) ax[k] *= force;
  if (j->body[0]) dBodyAddForce(j->body[0], ax[0], ax[1], ax[2]);
  if (j->body[1]) dBodyAddForce(j->body[1], -ax[0], -ax[1], -ax[2]);
  if (j->body[0] && j->body[1]) {
    dReal c[3], ltd[3];
    for (int k = 0; k < 3; ++k) c[k] = (dReal)0.5 * (j->body[1]->pos[k] - j->body[0]->pos[k]);
    ltd[0] = c[1] * ax[2] - c[2] * ax[1];
    ltd[1] = c[2] * ax[0] - c[0] * ax[2];
    ltd[2] = c[0] * ax[1] - c[1] * ax[0];
    dBodyAddTorque(j->body[0], ltd[0], ltd[1], ltd[2]);
    dBodyAddTorque(j->body[1], ltd[0], ltd[1], ltd[2]);
  }
}

// universal (ode/src/joints/universal.cpp)
void dJointSetUniversalAnchor(dJointID j, dReal x, dReal y, dReal z) {
  // :396-403
  JB jb(j);
  og_host::set_anchors(j->h, jb.B, x, y, z, j->h.anchor1, j->h.anchor2);
  og_host::universal_qrels(j->h, jb.B);
}
void dJointSetUniversalAxis1(dJointID j, dReal x, dReal y, dReal z) {
  // :406-415: on a reversed joint axis 1 is body 2's axis
  JB jb(j);
  if (j->reverse) og_host::set_axes(j->h, jb.B, x, y, z, nullptr, j->h.axis2);
  else og_host::set_axes(j->h, jb.B, x, y, z, j->h.axis1, nullptr);
  og_host::universal_qrels(j->h, jb.B);
}
void dJointSetUniversalAxis2(dJointID j, dReal x, dReal y, dReal z) {
  // :481-490
  JB jb(j);
  if (j->reverse) og_host::set_axes(j->h, jb.B, x, y, z, j->h.axis1, nullptr);
  else og_host::set_axes(j->h, jb.B, x, y, z, nullptr, j->h.axis2);
  og_host::universal_qrels(j->h, jb.B);
}
void dJointGetUniversalAnchor(dJointID j, dVector3 r) {
  // :559-569 (a reversed joint reports the body-2 anchor, which it lacks)
  if (j->reverse) return;
  double a[3];
  if (j->body[0]) { world_anchor1(j, a); for (int k = 0; k < 3; ++k) r[k] = (dReal)a[k]; }
}
void dJointGetUniversalAxis1(dJointID j, dVector3 r) {
  if (j->reverse) world_axis2(j, j->h.axis2, r); else world_axis1(j, j->h.axis1, r);
}
void dJointGetUniversalAxis2(dJointID j, dVector3 r) {
  if (j->reverse) world_axis1(j, j->h.axis1, r); else world_axis2(j, j->h.axis2, r);
}
void dJointSetUniversalParam(dJointID j, int p, dReal v) {
  // :611-624
  if ((p & 0xff00) == 0x100) limot_set(j->lm2, p & 0xff, v);
  else limot_set(j->lm1, p, v);
}
dReal dJointGetUniversalParam(dJointID j, int p) {
  if ((p & 0xff00) == 0x100) return limot_get(j->lm2, p & 0xff);
  return limot_get(j->lm1, p);
}
void dJointGetUniversalAngles(dJointID j, dReal* angle1, dReal* angle2) {
  // :642-655
  JB jb(j);
  double a1 = 0, a2 = 0;
  if (j->body[0]) og_host::universal_angles(j->h, jb.B, &a1, &a2);
  if (j->reverse) { *angle1 = (dReal)a2; *angle2 = (dReal)-a1; }
  else { *angle1 = (dReal)a1; *angle2 = (dReal)a2; }
}
dReal dJointGetUniversalAngle1(dJointID j) {
  // :658-667
  if (!j->body[0]) return 0;
  JB jb(j);
  return (dReal)(j->reverse ? og_host::universal_angle2(j->h, jb.B) : og_host::universal_angle1(j->h, jb.B));
}
dReal dJointGetUniversalAngle2(dJointID j) {
  // :670-679
  if (!j->body[0]) return 0;
  JB jb(j);
  return (dReal)(j->reverse ? -og_host::universal_angle1(j->h, jb.B) : og_host::universal_angle2(j->h, jb.B));
}
// Angle rates (ode/src/joints/hinge2.cpp:357-390, universal.cpp:682-726): the
// world axis dotted with the bodies' angular velocities. The hinge2 rates read
// the bodies as attached, without the reversal the angles apply.
static double joint_rate(const dxJoint* j, const double* ax) {
  const dReal* w0 = j->body[0]->avel;
  double rate = ax[0] * w0[0] + ax[1] * w0[1] + ax[2] * w0[2];
  if (j->body[1]) {
    const dReal* w1 = j->body[1]->avel;
    rate -= ax[0] * w1[0] + ax[1] * w1[1] + ax[2] * w1[2];
  }
  return rate;
}
static void body_axis(const dxBody* b, const double* axis, double* out) {   // R axis
  double R[12];
  for (int k = 0; k < 12; ++k) R[k] = b->R[k];
  og_host::mul0_331(out, R, axis);
}
static void axis2_world(const dxJoint* j, double* out) {   // getAxis2 (joint.cpp)
  if (j->body[1]) body_axis(j->body[1], j->h.axis2, out);
  else for (int k = 0; k < 3; ++k) out[k] = j->h.axis2[k];
}
dReal dJointGetHinge2Angle1Rate(dJointID j) {
  if (!j->body[0]) return 0;
  double ax[3];
  body_axis(j->body[0], j->h.axis1, ax);
  return (dReal)joint_rate(j, ax);
}
dReal dJointGetHinge2Angle2Rate(dJointID j) {
  if (!j->body[0] || !j->body[1]) return 0;
  double ax[3];
  body_axis(j->body[1], j->h.axis2, ax);
  return (dReal)joint_rate(j, ax);
}
dReal dJointGetUniversalAngle1Rate(dJointID j) {
  if (!j->body[0]) return 0;
  double ax[3];
  if (j->reverse) axis2_world(j, ax);
  else body_axis(j->body[0], j->h.axis1, ax);
  return (dReal)joint_rate(j, ax);
}
dReal dJointGetUniversalAngle2Rate(dJointID j) {
  if (!j->body[0]) return 0;
  double ax[3];
  if (j->reverse) body_axis(j->body[0], j->h.axis1, ax);
  else axis2_world(j, ax);
  return (dReal)joint_rate(j, ax);
}
// dQFromAxisAndAngle (rotation.cpp:169-189) in FP64, for the setters below
static void q_from_axis_angle(double* q, double ax, double ay, double az, double angle) {
  double l = ax * ax + ay * ay + az * az;
  if (l > 0) {
    angle *= 0.5;
    q[0] = std::cos(angle);
    l = std::sin(angle) / std::sqrt(l);
    q[1] = ax * l; q[2] = ay * l; q[3] = az * l;
  } else {
    q[0] = 1; q[1] = q[2] = q[3] = 0;
  }
}
// dJointSetUniversalAxis1Offset / Axis2Offset (universal.cpp:418-556): set the
// axis, then the relative rotations that make the current pose read the given
// angles. As in the reference: the second offset is composed with
// dQMultiply1, and on a reversed joint Axis2Offset's swap leaves offset2 as
// given (offset1 = -offset2 is assigned first).
static void universal_offset_qrels(dxJoint* j, const double* a1, const double* a2, double off1, double off2) {
  JB jb(j);
  double qa[4], R[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, qc[4], qo[4];
  q_from_axis_angle(qa, a1[0], a1[1], a1[2], off1);
  og_host::r_from_2axes(R, a1[0], a1[1], a1[2], a2[0], a2[1], a2[2]);
  og_host::q_from_r(qc, R);
  og_host::qmul0(qo, qa, qc);
  og_host::qmul1(j->h.qrel, jb.B[0].q, qo);
  q_from_axis_angle(qa, a2[0], a2[1], a2[2], off2);
  og_host::r_from_2axes(R, a2[0], a2[1], a2[2], a1[0], a1[1], a1[2]);
  og_host::q_from_r(qc, R);
  og_host::qmul1(qo, qa, qc);
  if (j->body[1]) og_host::qmul1(j->h.qrel2, jb.B[1].q, qo);
  else for (int k = 0; k < 4; ++k) j->h.qrel2[k] = qc[k];
}
void dJointSetUniversalAxis1Offset(dJointID j, dReal x, dReal y, dReal z, dReal offset1, dReal offset2) {
  JB jb(j);
  if (j->reverse) {
    og_host::set_axes(j->h, jb.B, x, y, z, nullptr, j->h.axis2);
    offset1 = -offset1;
    offset2 = -offset2;
  } else {
    og_host::set_axes(j->h, jb.B, x, y, z, j->h.axis1, nullptr);
  }
  og_host::universal_qrels(j->h, jb.B);
  if (!j->body[0]) return;
  double ax2[3];
  axis2_world(j, ax2);
  const double a1[3] = {x, y, z};
  universal_offset_qrels(j, a1, ax2, offset1, offset2);
}
void dJointSetUniversalAxis2Offset(dJointID j, dReal x, dReal y, dReal z, dReal offset1, dReal offset2) {
  JB jb(j);
  if (j->reverse) {
    og_host::set_axes(j->h, jb.B, x, y, z, j->h.axis1, nullptr);
    offset1 = -offset2;
    offset2 = -offset1;
  } else {
    og_host::set_axes(j->h, jb.B, x, y, z, nullptr, j->h.axis2);
  }
  og_host::universal_qrels(j->h, jb.B);
  if (!j->body[0]) return;
  double ax1[3], ax2[3];
  og_host::universal_axes(j->h, jb.B, ax1, ax2);
  universal_offset_qrels(j, ax1, ax2, offset1, offset2);
}
// dJointSetBallAnchor2 (ball.cpp:79-88): body 2's anchor as given, untransformed
void dJointSetBallAnchor2(dJointID j, dReal x, dReal y, dReal z) {
  j->h.anchor2[0] = x; j->h.anchor2[1] = y; j->h.anchor2[2] = z; j->h.anchor2[3] = 0;
}
// dJointSetHingeAnchorDelta (hinge.cpp:163-199): as dJointSetHingeAnchor, but
// a hinge to the environment keeps anchor + delta as its fixed point
void dJointSetHingeAnchorDelta(dJointID j, dReal x, dReal y, dReal z, dReal dx, dReal dy, dReal dz) {
  JB jb(j);
  og_host::set_anchors(j->h, jb.B, x, y, z, j->h.anchor1, j->h.anchor2);
  if (j->body[0] && !j->body[1]) {
    const dReal p[3] = {x + dx, y + dy, z + dz};
    for (int k = 0; k < 3; ++k) j->h.anchor2[k] = p[k];
  }
  j->h.anchor1[3] = j->h.anchor2[3] = 0;
  og_host::hinge_qrel(j->h, jb.B);
}
// dJointSetHingeAxisOffset (hinge.cpp:213-230): the axis, then the relative
// rotation turned so that the current pose reads the given angle
void dJointSetHingeAxisOffset(dJointID j, dReal x, dReal y, dReal z, dReal dangle) {
  JB jb(j);
  og_host::set_axes(j->h, jb.B, x, y, z, j->h.axis1, j->h.axis2);
  og_host::hinge_qrel(j->h, jb.B);
  if (j->reverse) dangle = -dangle;
  double qa[4], qo[4];
  q_from_axis_angle(qa, x, y, z, dangle);
  og_host::qmul3(qo, qa, j->h.qrel);
  for (int k = 0; k < 4; ++k) j->h.qrel[k] = qo[k];
}
// dJointSetSliderAxisDelta (slider.cpp:243-262): as dJointSetSliderAxis, with
// a slider to the environment moving its reference point by the delta
void dJointSetSliderAxisDelta(dJointID j, dReal x, dReal y, dReal z, dReal dx, dReal dy, dReal dz) {
  JB jb(j);
  og_host::set_axes(j->h, jb.B, x, y, z, j->h.axis1, nullptr);
  og_host::slider_offset(j->h, jb.B);
  if (!j->body[1]) {
    j->h.offset[0] += dx; j->h.offset[1] += dy; j->h.offset[2] += dz;
  }
  og_host::initial_qrel(j->h, jb.B);
}
void dJointAddUniversalTorques(dJointID j, dReal t1, dReal t2) {
  // :729-754
  if (j->reverse) { const dReal tmp = t1; t1 = -t2; t2 = -tmp; }
  dVector3 a1 = {0, 0, 0, 0}, a2 = {0, 0, 0, 0};
  world_axis1(j, j->h.axis1, a1);
  world_axis2(j, j->h.axis2, a2);
  for (int k = 0; k < 3; ++k) a1[k] = a1[k] * t1 + a2[k] * t2;
  if (j->body[0]) dBodyAddTorque(j->body[0], a1[0], a1[1], a1[2]);
  if (j->body[1]) dBodyAddTorque(j->body[1], -a1[0], -a1[1], -a1[2]);
}

// fixed (ode/src/joints/fixed.cpp)
void dJointSetFixed(dJointID j) {
  // :110-132
  JB jb(j);
  og_host::fixed_offset(j->h, jb.B);
  og_host::initial_qrel(j->h, jb.B);
}
void dJointSetFixedParam(dJointID j, int p, dReal v) {
  if (p == dParamCFM) j->cfm = v; else if (p == dParamERP) j->erp = v;
}
dReal dJointGetFixedParam(dJointID j, int p) {
  if (p == dParamCFM) return (dReal)j->cfm;
  if (p == dParamERP) return (dReal)j->erp;
  return 0;
}

// angular motor (ode/src/joints/amotor.cpp)
void dJointSetAMotorNumAxes(dJointID j, int num) { og_host::amotor_set_num(j->h, num); }
void dJointSetAMotorAxis(dJointID j, int anum, int rel, dReal x, dReal y, dReal z) {
  JB jb(j);
  og_host::amotor_set_axis(j->h, jb.B, anum, rel, x, y, z);
}
void dJointSetAMotorAngle(dJointID j, int anum, dReal angle) {
  // :326-336 (user mode only)
  if (j->h.am_mode == dAMotorUser && anum >= 0 && anum < 3) j->h.am_angle[anum] = angle;
}
static og::DevLimot& amotor_limot(dJointID j, int parameter) {
  const int anum = std::min(2, std::max(0, parameter >> 8));
  return anum == 0 ? j->lm1 : anum == 1 ? j->lm2 : j->lm3;
}
void dJointSetAMotorParam(dJointID j, int p, dReal v) { limot_set(amotor_limot(j, p), p & 0xff, v); }
dReal dJointGetAMotorParam(dJointID j, int p) { return limot_get(amotor_limot(j, p), p & 0xff); }
void dJointSetAMotorMode(dJointID j, int mode) {
  JB jb(j);
  og_host::amotor_set_mode(j->h, jb.B, mode);
}
int dJointGetAMotorMode(dJointID j) { return j->h.am_mode; }
int dJointGetAMotorNumAxes(dJointID j) { return j->h.am_num; }
int dJointGetAMotorAxisRel(dJointID j, int anum) { return j->h.am_rel[std::min(2, std::max(0, anum))]; }
// the global axes (computeGlobalAxes, :52-94)
static void amotor_global_axes(const dxJoint* j, double ax[3][3]) {
  JB jb(j);
  const og_host::HJoint& H = j->h;
  const og_host::HBody* B2 = j->body[1] ? &jb.B[1] : nullptr;
  if (H.am_mode == dAMotorEuler) {
    og_host::mul0_331(ax[0], jb.B[0].R, H.am_axis[0]);
    if (B2) og_host::mul0_331(ax[2], B2->R, H.am_axis[2]);
    else for (int k = 0; k < 3; ++k) ax[2][k] = H.am_axis[2][k];
    og_host::cross3(ax[1], ax[2], ax[0]);
    og_host::safe_normalize3(ax[1]);
    return;
  }
  for (int i = 0; i < H.am_num; ++i) {
    if (H.am_rel[i] == 1) og_host::mul0_331(ax[i], jb.B[0].R, H.am_axis[i]);
    else if (H.am_rel[i] == 2 && B2) og_host::mul0_331(ax[i], B2->R, H.am_axis[i]);
    else for (int k = 0; k < 3; ++k) ax[i][k] = H.am_axis[i][k];
  }
}
void dJointGetAMotorAxis(dJointID j, int anum, dVector3 r) {
  // :393-420
  anum = std::min(2, std::max(0, anum));
  const og_host::HJoint& H = j->h;
  if (H.am_rel[anum] == 1) world_axis1(j, H.am_axis[anum], r);
  else if (H.am_rel[anum] == 2) world_axis2(j, H.am_axis[anum], r);
  else for (int k = 0; k < 3; ++k) r[k] = (dReal)H.am_axis[anum][k];
}
// ODE 0.12 leaves this unimplemented (amotor.cpp:445-451 stops in dDebug);
// here it answers 0
dReal dJointGetAMotorAngleRate(dJointID, int) { return 0; }
dReal dJointGetAMotorAngle(dJointID j, int anum) {
  // user mode: the angle set; Euler mode: the angles of the bodies' current
  // placement (the reference returns those its last getInfo1 computed)
  anum = std::min(2, std::max(0, anum));
  const og_host::HJoint& H = j->h;
  if (H.am_mode != dAMotorEuler || !j->body[0]) return (dReal)H.am_angle[anum];
  double ax[3][3], ref1[3], ref2[3], q[3];
  amotor_global_axes(j, ax);
  JB jb(j);
  og_host::mul0_331(ref1, jb.B[0].R, H.am_ref1);
  if (j->body[1]) og_host::mul0_331(ref2, jb.B[1].R, H.am_ref2);
  else for (int k = 0; k < 3; ++k) ref2[k] = H.am_ref2[k];
  if (anum == 0) {
    og_host::cross3(q, ax[0], ref1);
    return (dReal)-std::atan2(og_host::dot3(ax[2], q), og_host::dot3(ax[2], ref1));
  }
  if (anum == 1) {
    og_host::cross3(q, ax[0], ax[1]);
    return (dReal)-std::atan2(og_host::dot3(ax[2], ax[0]), og_host::dot3(ax[2], q));
  }
  og_host::cross3(q, ax[1], ax[2]);
  return (dReal)-std::atan2(og_host::dot3(ref2, ax[1]), og_host::dot3(ref2, q));
}
void dJointAddAMotorTorques(dJointID j, dReal t1, dReal t2, dReal t3) {
  // :474-504
  if (j->h.am_num == 0 || !j->body[0]) return;
  double ax[3][3];
  amotor_global_axes(j, ax);
  dReal t[3];
  for (int k = 0; k < 3; ++k) t[k] = (dReal)ax[0][k] * t1;
  if (j->h.am_num >= 2) {
    for (int k = 0; k < 3; ++k) t[k] += (dReal)ax[1][k] * t2;
    if (j->h.am_num >= 3) for (int k = 0; k < 3; ++k) t[k] += (dReal)ax[2][k] * t3;
  }
  dBodyAddTorque(j->body[0], t[0], t[1], t[2]);
  if (j->body[1]) dBodyAddTorque(j->body[1], -t[0], -t[1], -t[2]);
}

int dAreConnectedExcluding(dBodyID b1, dBodyID b2, int joint_type) {
  // ode/src/ode.cpp:1529-1537
  if (!b1) return 0;
  for (dxJoint* j : b1->world->joints) {
    if (j->type == joint_type) continue;
    if ((j->body[0] == b1 && j->body[1] == b2) || (j->body[1] == b1 && j->body[0] == b2)) return 1;
  }
  return 0;
}

// ---------------------------------------------------------------- RNG
int dTestRand(void) {
  unsigned long old = g_seed;
  int ok = 1;
  g_seed = 0;
  const unsigned long expect[5] = {0x3c6ef35f, 0x47502932, 0xd1ccf6e9, 0xaaf95334, 0x6252e503};
  for (int i = 0; i < 5; ++i) if (dRand() != expect[i]) ok = 0;
  g_seed = old;
  return ok;
}
unsigned long dRand(void) {
  g_seed = og::lcg_next((unsigned)g_seed);
  return g_seed;
}
unsigned long dRandGetSeed(void) { return g_seed; }
void dRandSetSeed(unsigned long s) { g_seed = s & 0xffffffffUL; }
int dRandInt(int n) { return og::rand_int_from((unsigned)dRand(), n); }

// ---------------------------------------------------------------- geoms + dCollide
// ---------------------------------------------------------------- spaces (core)
// The list discipline of collision_space.cpp:42-206: a geom joins its space at
// the front; a clean geom that moves becomes dirty and goes to the front again,
// and so do its parent spaces; dSpaceCollide cleans the dirty prefix (boxes
// recomputed, flags cleared) and then visits pairs in list order. The order of
// the near-callback's pairs, and with it the order of the contact joints a
// program creates, follows from this.
static void list_push_front(dxGeom** first, dxGeom* g) {   // dxGeom::spaceAdd
  g->next = *first;
  g->tome = first;
  if (*first) (*first)->tome = &g->next;
  *first = g;
}
static void list_unlink(dxGeom* g) {   // dxGeom::spaceRemove
  if (g->next) g->next->tome = g->tome;
  *g->tome = g->next;
}
// dxSAPSpace::dirty (collision_sapspace.cpp:363-387): from the clean list
// (the last one takes its slot) to the end of the dirty list
static void sap_dirty(SapSpace& S, dxGeom* g) {
  if (g->sap_dirty >= 0) return;
  const int gi = g->sap_clean;
  dxGeom* last = S.geoms.back();
  S.geoms[gi] = last;
  last->sap_clean = gi;
  S.geoms.pop_back();
  g->sap_clean = -1;
  g->sap_dirty = (int)S.dirty.size();
  S.dirty.push_back(g);
}
// dGeomMoved (collision_space.cpp:47-74)
static void geom_moved(dxGeom* g) {
  dxSpace* parent = g->space;
  while (parent && !g->dirty) {
    g->dirty = g->aabb_bad = 1;
    if (parent->qt) {
      parent->qt->dirty.push_back(g);   // dxQuadTreeSpace::dirty
    } else if (parent->sap) {
      sap_dirty(*parent->sap, g);
    } else {
      list_unlink(g);
      list_push_front(&parent->first, g);
    }
    g = parent;
    parent = parent->space;
  }
  for (; g; g = g->space) g->dirty = g->aabb_bad = 1;
}
// Block::Inside / GetBlock / GetBlockChild / AddObject / DelObject
// (collision_quadtreespace.cpp:251-331)
static bool quad_inside(const QuadBlock& b, const dReal* a) {
  return a[0] >= b.minx && a[1] < b.maxx && a[2] >= b.miny && a[3] < b.maxy;
}
static int quad_block_child(const QuadTree& q, int b, const dReal* a) {
  for (;;) {
    const int c = q.blocks[b].children;
    if (c < 0) return b;
    int next = -1;
    for (int i = 0; i < 4 && next < 0; ++i)
      if (quad_inside(q.blocks[c + i], a)) next = c + i;
    if (next < 0) return b;
    b = next;
  }
}
static int quad_block(const QuadTree& q, int b, const dReal* a) {
  for (;;) {
    if (quad_inside(q.blocks[b], a)) return quad_block_child(q, b, a);
    if (q.blocks[b].parent < 0) return b;
    b = q.blocks[b].parent;
  }
}
static void quad_add(QuadTree& q, int b, dxGeom* g) {
  g->next = q.blocks[b].first;
  q.blocks[b].first = g;
  g->qblock = b;
  for (int k = b; k >= 0; k = q.blocks[k].parent) ++q.blocks[k].count;
}
static void quad_del(QuadTree& q, dxGeom* g) {
  const int b = g->qblock;
  for (dxGeom** l = &q.blocks[b].first; *l; l = &(*l)->next)
    if (*l == g) { *l = g->next; break; }
  g->qblock = -1;
  for (int k = b; k >= 0; k = q.blocks[k].parent) --q.blocks[k].count;
}

// dxSpace::add / remove (collision_space.cpp:162-206, quadtree :485-532)
static void space_add(dxSpace* s, dxGeom* g) {
  if (!s || !g || g->space) return;
  if (s->sap) {   // dxSAPSpace::add (:303-320)
    g->dirty = g->aabb_bad = 1;
    g->sap_dirty = (int)s->sap->dirty.size();
    g->sap_clean = -1;
    s->sap->dirty.push_back(g);
    g->space = s;
    ++s->count;
    geom_moved(s);
    return;
  }
  if (s->qt) {
    g->dirty = g->aabb_bad = 1;
    s->qt->dirty.push_back(g);
    g->space = s;
    quad_add(*s->qt, quad_block(*s->qt, 0, g->aabb), g);   // by the box it has now
    ++s->count;
    geom_moved(s);
    return;
  }
  g->space = s;
  list_push_front(&s->first, g);
  ++s->count;
  g->dirty = g->aabb_bad = 1;
  geom_moved(s);
}
static void space_remove(dxSpace* s, dxGeom* g) {
  if (!s || !g || g->space != s) return;
  if (s->sap) {   // dxSAPSpace::remove (:322-361)
    SapSpace& S = *s->sap;
    if (g->sap_dirty >= 0) {
      dxGeom* last = S.dirty.back();
      S.dirty[g->sap_dirty] = last;
      last->sap_dirty = g->sap_dirty;
      S.dirty.pop_back();
    } else {
      dxGeom* last = S.geoms.back();
      S.geoms[g->sap_clean] = last;
      last->sap_clean = g->sap_clean;
      S.geoms.pop_back();
    }
    g->sap_dirty = g->sap_clean = -1;
    --s->count;
    g->space = nullptr;
    geom_moved(s);
    return;
  }
  if (s->qt) {
    quad_del(*s->qt, g);
    --s->count;
    auto& d = s->qt->dirty;
    d.erase(std::remove(d.begin(), d.end(), g), d.end());
    g->next = nullptr;
    g->space = nullptr;
    geom_moved(s);
    return;
  }
  list_unlink(g);
  --s->count;
  g->next = nullptr;
  g->tome = nullptr;
  g->space = nullptr;
  geom_moved(s);
}
static void body_list_remove(dxGeom* g) {   // dxGeom::bodyRemove (collision_kernel.cpp:396-412)
  if (!g->body) return;
  for (dxGeom** l = &g->body->geom; *l; l = &(*l)->body_next)
    if (*l == g) { *l = g->body_next; break; }
  g->body = nullptr;
  g->body_next = nullptr;
}
static void body_geoms_moved(dxBody* b) {
  for (dxGeom* g = b->geom; g; g = g->body_next) geom_moved(g);
}
static void body_geoms_detach(dxBody* b) {   // dBodyDestroy (ode.cpp:301-310)
  for (dxGeom *g = b->geom, *n; g; g = n) {
    n = g->body_next;
    dGeomSetBody(g, nullptr);
  }
}

// dxGeom::dxGeom (collision_kernel.cpp:343-368): identity pose, enabled,
// dirty, all category and collide bits set, then into the space if one is given
static void init_geom(dxGeom* g, dSpaceID space, int type) {
  g->type = type;
  g->R[0] = g->R[5] = g->R[10] = 1;
  g->category_bits = g->collide_bits = ~0UL;
  g->enabled = 1;
  g->dirty = g->aabb_bad = 1;
  if (space) space_add(space, g);
}
static dGeomID new_geom(dSpaceID space, int type, const double* p) {
  auto* g = new dxGeom();
  std::memset(g, 0, sizeof(*g));
  for (int k = 0; k < 4; ++k) g->p[k] = p[k];
  // GEOM_ZERO_SIZED (sphere.cpp:55, box.cpp:56, capsule.cpp:56, cylinder.cpp:55)
  if (type == dSphereClass || type == dCapsuleClass) g->zero_sized = (dReal)p[0] == 0;
  if (type == dBoxClass) g->zero_sized = (dReal)p[0] == 0 || (dReal)p[1] == 0 || (dReal)p[2] == 0;
  if (type == dCylinderClass) g->zero_sized = (dReal)p[0] == 0 || (dReal)p[1] == 0;
  init_geom(g, space, type);
  return g;
}
dGeomID dCreateSphere(dSpaceID s, dReal r) { const double p[4] = {r, 0, 0, 0}; return new_geom(s, dSphereClass, p); }
dGeomID dCreateBox(dSpaceID s, dReal lx, dReal ly, dReal lz) {
  const double p[4] = {lx, ly, lz, 0};
  return new_geom(s, dBoxClass, p);
}
dGeomID dCreateCapsule(dSpaceID s, dReal r, dReal len) {
  const double p[4] = {r, len, 0, 0};
  return new_geom(s, dCapsuleClass, p);
}
dGeomID dCreateCylinder(dSpaceID s, dReal r, dReal len) {
  const double p[4] = {r, len, 0, 0};
  return new_geom(s, dCylinderClass, p);
}
void dGeomCylinderSetParams(dGeomID g, dReal r, dReal len) {   // cylinder.cpp:84-93
  if (!g || g->type != dCylinderClass) return;
  g->p[0] = r; g->p[1] = len;
  g->zero_sized = r == 0 || len == 0;
  geom_moved(g);
}
void dGeomCylinderGetParams(dGeomID g, dReal* r, dReal* l) {
  if (g && g->type == dCylinderClass) { *r = (dReal)g->p[0]; *l = (dReal)g->p[1]; }
}
// make_sure_plane_normal_has_unit_length (ode/src/plane.cpp:49-65), in dReal
// arithmetic as the dSINGLE build does it
static void plane_params(double* p, dReal a, dReal b, dReal c, dReal d) {
  dReal q[4] = {a, b, c, d};
  dReal l = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
  if (l > 0) { l = (dReal)1 / std::sqrt(l); for (int k = 0; k < 4; ++k) q[k] *= l; }
  else { q[0] = 1; q[1] = q[2] = q[3] = 0; }
  for (int k = 0; k < 4; ++k) p[k] = q[k];
}
dGeomID dCreatePlane(dSpaceID s, dReal a, dReal b, dReal c, dReal d) {
  double p[4];
  plane_params(p, a, b, c, d);
  return new_geom(s, dPlaneClass, p);
}
// dGeomDestroy (collision_kernel.cpp:486-490 with ~dxGeom, :376-383): a space
// first destroys (cleanup on) or releases its geoms (collision_space.cpp:96-113);
// then the geom leaves its space and its body
void dGeomDestroy(dGeomID g) {
  if (!g) return;
  if (is_space(g)) {
    auto* sp = static_cast<dxSpace*>(g);
    for (dxGeom *c = sp->first, *n; c; c = n) {
      n = c->next;
      if (sp->cleanup) dGeomDestroy(c);
      else space_remove(sp, c);
    }
    if (sp->sap) {
      // ~dxSAPSpace (:278-291): the first of each list until it is empty
      SapSpace& S = *sp->sap;
      for (std::vector<dxGeom*>* l : {&S.dirty, &S.geoms})
        while (!l->empty()) {
          if (sp->cleanup) dGeomDestroy((*l)[0]);
          else space_remove(sp, (*l)[0]);
        }
      delete sp->sap;
      sp->sap = nullptr;
    }
    if (sp->qt) {
      // ODE 0.12's space destructor walks the base list, which a quadtree
      // space leaves empty, so its geoms are neither destroyed nor released
      // there; here they are released
      for (QuadBlock& b : sp->qt->blocks)
        for (dxGeom *c = b.first, *n; c; c = n) {
          n = c->next;
          c->next = nullptr;
          c->qblock = -1;
          c->space = nullptr;
        }
      delete sp->qt;
      sp->qt = nullptr;
    }
  }
  if (g->type == dGeomTransformClass && g->tobj && g->tcleanup) dGeomDestroy(g->tobj);   // ~dxGeomTransform
  if (const dGeomClass* uc = user_class_of(g)) {   // ~dxUserGeom: the class's destructor, then its block
    if (uc->dtor) uc->dtor(g);
    std::free(g->class_data);
  }
  if (g->space) space_remove(g->space, g);
  body_list_remove(g);
  if (is_space(g)) delete static_cast<dxSpace*>(g);
  else delete g;
}

// Rays (ode/src/ray.cpp:49-194): the length is the class parameter; the start
// is the geom's position and the direction column 2 of its rotation, so a ray
// attached to a body follows that body.
dGeomID dCreateRay(dSpaceID s, dReal length) {
  const double p[4] = {length, 0, 0, 0};
  return new_geom(s, dRayClass, p);
}
void dGeomRaySetLength(dGeomID g, dReal length) {
  if (!g || g->type != dRayClass) return;
  g->p[0] = length;
  geom_moved(g);
}
dReal dGeomRayGetLength(dGeomID g) { return (g && g->type == dRayClass) ? (dReal)g->p[0] : 0; }
void dGeomRaySet(dGeomID g, dReal px, dReal py, dReal pz, dReal dx, dReal dy, dReal dz) {
  // writes the placement the ray reads: a body's own when attached
  // (final_posr is the body's, ray.cpp:115-136), with the direction normalised
  // An offset ray writes its own final pose, which the next read rebuilds
  // from the body and the offset (ray.cpp:113-135 with dGeomMoved), so the
  // call changes nothing there.
  if (!g || g->type != dRayClass) return;
  if (!g->has_offset) {
    double n[3] = {dx, dy, dz};
    og_host::safe_normalize3(n);
    dReal* pos = g->body ? g->body->pos : g->pos;
    dReal* R = g->body ? g->body->R : g->R;
    pos[0] = px; pos[1] = py; pos[2] = pz;
    R[2] = (dReal)n[0]; R[6] = (dReal)n[1]; R[10] = (dReal)n[2];
  }
  geom_moved(g);
}
void dGeomRayGet(dGeomID g, dVector3 start, dVector3 dir) {
  if (!g || g->type != dRayClass) return;
  const dReal* pos = dGeomGetPosition(g);
  const dReal* R = dGeomGetRotation(g);
  for (int k = 0; k < 3; ++k) { start[k] = pos[k]; dir[k] = R[k * 4 + 2]; }
}
void dGeomRaySetParams(dGeomID g, int FirstContact, int BackfaceCull) {
  if (!g || g->type != dRayClass) return;
  g->ray_flags = (g->ray_flags & kRayClosestHit) | (FirstContact ? kRayFirstContact : 0) |
                 (BackfaceCull ? kRayBackfaceCull : 0);
}
void dGeomRayGetParams(dGeomID g, int* FirstContact, int* BackfaceCull) {
  if (!g || g->type != dRayClass) return;
  *FirstContact = (g->ray_flags & kRayFirstContact) != 0;
  *BackfaceCull = (g->ray_flags & kRayBackfaceCull) != 0;
}
void dGeomRaySetClosestHit(dGeomID g, int closestHit) {
  if (!g || g->type != dRayClass) return;
  g->ray_flags = closestHit ? (g->ray_flags | kRayClosestHit) : (g->ray_flags & ~kRayClosestHit);
}
int dGeomRayGetClosestHit(dGeomID g) { return (g && g->type == dRayClass && (g->ray_flags & kRayClosestHit)) ? 1 : 0; }

// Heightfields (ode/src/heightfield.cpp:107-143, :1860-2000): the samples are
// copied at build time whatever bCopyHeightData says, and uploaded to the GPU.
dHeightfieldDataID dGeomHeightfieldDataCreate(void) { return new dxHeightfieldData(); }
void dGeomHeightfieldDataDestroy(dHeightfieldDataID d) {
  if (!d) return;
  og::free_heights(d->d_heights);
  delete d;
}
static bool hf_shape(dHeightfieldDataID d, dReal width, dReal depth, int widthSamples, int depthSamples,
                     dReal scale, dReal offset, dReal thickness, int bWrap) {
  if (!d || widthSamples < 2 || depthSamples < 2 || !(width > 0) || !(depth > 0)) return false;
  d->nx = widthSamples; d->nz = depthSamples; d->wrap = bWrap;
  d->width = width; d->depth = depth; d->scale = scale; d->offset = offset; d->thickness = thickness;
  d->heights.assign((size_t)widthSamples * depthSamples, 0.f);
  return true;
}
// dxHeightfieldData::ComputeHeightBounds (heightfield.cpp:150-237) over the
// samples as dReal, then scale, offset and thickness
static void hf_bounds(dHeightfieldDataID d) {
  float lo = INFINITY, hi = -INFINITY;
  for (const float h : d->heights) {
    if (h < lo) lo = h;
    if (h > hi) hi = h;
  }
  const float sc = (float)d->scale, of = (float)d->offset, th = (float)d->thickness;
  lo *= sc; hi *= sc;
  lo += of; hi += of;
  lo -= th;
  d->hmin = lo; d->hmax = hi;
}
void dGeomHeightfieldDataBuildSingle(dHeightfieldDataID d, const float* pHeightData, int, dReal width,
                                     dReal depth, int widthSamples, int depthSamples, dReal scale, dReal offset,
                                     dReal thickness, int bWrap) {
  if (!pHeightData || !hf_shape(d, width, depth, widthSamples, depthSamples, scale, offset, thickness, bWrap))
    return;
  for (size_t k = 0; k < d->heights.size(); ++k) d->heights[k] = pHeightData[k];
  hf_bounds(d);
  d->built = og::upload_heights(d->heights, &d->d_heights) == 0;
}
void dGeomHeightfieldDataBuildDouble(dHeightfieldDataID d, const double* pHeightData, int, dReal width,
                                     dReal depth, int widthSamples, int depthSamples, dReal scale, dReal offset,
                                     dReal thickness, int bWrap) {
  if (!pHeightData || !hf_shape(d, width, depth, widthSamples, depthSamples, scale, offset, thickness, bWrap))
    return;
  for (size_t k = 0; k < d->heights.size(); ++k) d->heights[k] = (float)pHeightData[k];
  hf_bounds(d);
  d->built = og::upload_heights(d->heights, &d->d_heights) == 0;
}
void dGeomHeightfieldDataBuildByte(dHeightfieldDataID d, const unsigned char* pHeightData, int, dReal width,
                                   dReal depth, int widthSamples, int depthSamples, dReal scale, dReal offset,
                                   dReal thickness, int bWrap) {
  if (!pHeightData || !hf_shape(d, width, depth, widthSamples, depthSamples, scale, offset, thickness, bWrap))
    return;
  for (size_t k = 0; k < d->heights.size(); ++k) d->heights[k] = (float)pHeightData[k];
  hf_bounds(d);
  d->built = og::upload_heights(d->heights, &d->d_heights) == 0;
}
// dGeomHeightfieldDataBuildCallback (heightfield.cpp:676-697): the callback
// is sampled here once for every sample and the field is then used like a
// built one (ODE calls it for the cells each collision touches, so a callback
// whose answers change later is not followed). Its bounds are infinite until
// dGeomHeightfieldDataSetBounds.
void dGeomHeightfieldDataBuildCallback(dHeightfieldDataID d, void* pUserData, dHeightfieldGetHeight* pCallback,
                                       dReal width, dReal depth, int widthSamples, int depthSamples, dReal scale,
                                       dReal offset, dReal thickness, int bWrap) {
  if (!pCallback || !hf_shape(d, width, depth, widthSamples, depthSamples, scale, offset, thickness, bWrap)) return;
  for (int z = 0; z < depthSamples; ++z)
    for (int x = 0; x < widthSamples; ++x) d->heights[(size_t)z * widthSamples + x] = pCallback(pUserData, x, z);
  d->hmin = -INFINITY;
  d->hmax = INFINITY;
  d->built = og::upload_heights(d->heights, &d->d_heights) == 0;
}
void dGeomHeightfieldDataBuildShort(dHeightfieldDataID d, const short* pHeightData, int, dReal width, dReal depth,
                                    int widthSamples, int depthSamples, dReal scale, dReal offset, dReal thickness,
                                    int bWrap) {
  if (!pHeightData || !hf_shape(d, width, depth, widthSamples, depthSamples, scale, offset, thickness, bWrap))
    return;
  for (size_t k = 0; k < d->heights.size(); ++k) d->heights[k] = (float)pHeightData[k];
  hf_bounds(d);
  d->built = og::upload_heights(d->heights, &d->d_heights) == 0;
}
// The bounds set the field's vertical extent in its bounding box
// (heightfield.cpp:845-850), which dGeomGetAABB reports and only a space's
// early rejection would read; dCollide does not.
void dGeomHeightfieldDataSetBounds(dHeightfieldDataID d, dReal minHeight, dReal maxHeight) {
  if (!d) return;
  const float sc = (float)d->scale, of = (float)d->offset, th = (float)d->thickness;
  d->hmin = minHeight * sc + of - th;
  d->hmax = maxHeight * sc + of;
}
// As in ODE 0.12 (heightfield.cpp:869-880), the setter stores the handle as
// the geom's user data and leaves the field it collides with unchanged.
void dGeomHeightfieldSetHeightfieldData(dGeomID g, dHeightfieldDataID d) { g->data = d; }
dHeightfieldDataID dGeomHeightfieldGetHeightfieldData(dGeomID g) { return g->hf; }
dGeomID dCreateHeightfield(dSpaceID s, dHeightfieldDataID data, int bPlaceable) {
  const double p[4] = {0, 0, 0, 0};
  dGeomID g = new_geom(s, dHeightfieldClass, p);
  g->hf = data;
  g->placeable = bPlaceable;
  return g;
}
// ---------------------------------------------------------------- geom placement
// A geom on a body reads the body's pose; with an offset it has its own final
// pose, body.R * offset.pos + body.pos and body.R * offset.R
// (dxGeom::computePosr, collision_kernel.cpp:454-465), recomputed on every read
// so that it follows the body through the step. Planes and non-placeable
// heightfields have no pose (GEOM_PLACEABLE clear).
static bool geom_placeable(const dxGeom* g) {
  return !is_space(g) && g->type != dPlaneClass && !(g->type == dHeightfieldClass && !g->placeable);
}
static void mul0_331(dReal* a, const dReal* R, const dReal* v) {   // a = R v
  for (int i = 0; i < 3; ++i) a[i] = R[i * 4 + 0] * v[0] + R[i * 4 + 1] * v[1] + R[i * 4 + 2] * v[2];
}
static void mul1_331(dReal* a, const dReal* R, const dReal* v) {   // a = R^T v
  for (int i = 0; i < 3; ++i) a[i] = R[0 * 4 + i] * v[0] + R[1 * 4 + i] * v[1] + R[2 * 4 + i] * v[2];
}
static void mul0_333(dReal* A, const dReal* B, const dReal* C) {   // A = B C, pads kept
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      A[i * 4 + j] = B[i * 4 + 0] * C[0 * 4 + j] + B[i * 4 + 1] * C[1 * 4 + j] + B[i * 4 + 2] * C[2 * 4 + j];
}
static void transpose33(dReal* T, const dReal* R) {   // matrixInvert (collision_kernel.cpp:417-426)
  for (int k = 0; k < 12; ++k) T[k] = R[k];
  std::swap(T[4], T[1]);
  std::swap(T[2], T[8]);
  std::swap(T[9], T[6]);
}
static void geom_recompute(dxGeom* g) {
  if (!g->has_offset || !g->body) return;
  mul0_331(g->fpos, g->body->R, g->opos);
  for (int k = 0; k < 3; ++k) g->fpos[k] += g->body->pos[k];
  mul0_333(g->fR, g->body->R, g->oR);
}
static dReal* geom_pos(dxGeom* g) {
  if (g->ovr_pos) return const_cast<dReal*>(g->ovr_pos);
  geom_recompute(g);
  return g->has_offset ? g->fpos : g->body ? g->body->pos : g->pos;
}
static dReal* geom_R(dxGeom* g) {
  if (g->ovr_R) return const_cast<dReal*>(g->ovr_R);
  geom_recompute(g);
  return g->has_offset ? g->fR : g->body ? g->body->R : g->R;
}
// dxGeomTransform::computeFinalTx (collision_transform.cpp:94-102): the
// wrapped geom's own pose carried by the transform's
static void transform_final(dxGeom* tr) {
  const dReal* R = geom_R(tr);
  const dReal* P = geom_pos(tr);
  const dReal* op = geom_pos(tr->tobj);
  mul0_331(tr->tpos, R, op);
  for (int k = 0; k < 3; ++k) tr->tpos[k] += P[k];
  mul0_333(tr->tR, R, geom_R(tr->tobj));
}
// getBodyPosr (collision_kernel.cpp:428-439): the body pose that puts the
// offset geom at (fpos, fR)
static void body_for_final(const dxGeom* g, const dReal* fpos, const dReal* fR, dReal* bpos, dReal* bR) {
  dReal inv[12], wo[3];
  transpose33(inv, g->oR);
  for (int k = 0; k < 12; ++k) bR[k] = 0;
  mul0_333(bR, fR, inv);
  mul0_331(wo, bR, g->opos);
  for (int k = 0; k < 3; ++k) bpos[k] = fpos[k] - wo[k];
}
// getWorldOffsetPosr (collision_kernel.cpp:441-452): the offset that puts the
// geom at (fpos, fR) on its body as it stands
static void offset_for_final(dxGeom* g, const dReal* fpos, const dReal* fR) {
  dReal inv[12], wo[3];
  transpose33(inv, g->body->R);
  mul0_333(g->oR, inv, fR);
  for (int k = 0; k < 3; ++k) wo[k] = fpos[k] - g->body->pos[k];
  mul0_331(g->opos, inv, wo);
}
// dGeomCreateOffset (collision_kernel.cpp:1017-1034): a zero offset
static bool geom_make_offset(dxGeom* g) {
  if (!g || !g->body || !geom_placeable(g)) return false;
  if (g->has_offset) return true;
  g->has_offset = 1;
  for (int k = 0; k < 4; ++k) g->opos[k] = 0;
  for (int k = 0; k < 12; ++k) g->oR[k] = 0;
  g->oR[0] = g->oR[5] = g->oR[10] = 1;
  return true;
}

// dGeomSetBody (collision_kernel.cpp:507-546): attaching to another body drops
// any offset; detaching keeps the geom where it was (its final pose, or the
// body's) as its own
void dGeomSetBody(dGeomID g, dBodyID b) {
  if (!g || !geom_placeable(g)) return;
  if (b) {
    if (g->body != b) {
      g->has_offset = 0;
      body_list_remove(g);
      g->body = b;
      g->body_next = b->geom;
      b->geom = g;
    }
    geom_moved(g);
  } else if (g->body) {
    const dReal* pos = geom_pos(g);
    const dReal* R = geom_R(g);
    for (int k = 0; k < 3; ++k) g->pos[k] = pos[k];
    for (int k = 0; k < 12; ++k) g->R[k] = R[k];
    g->has_offset = 0;
    body_list_remove(g);
  }
}
dBodyID dGeomGetBody(dGeomID g) { return g->body; }
// dGeomSetPosition / SetRotation / SetQuaternion (collision_kernel.cpp:557-640):
// an offset geom moves its body so that body + offset lands on the new pose
void dGeomSetPosition(dGeomID g, dReal x, dReal y, dReal z) {
  if (g->has_offset) {
    dReal wo[3];
    mul0_331(wo, g->body->R, g->opos);
    dBodySetPosition(g->body, x - wo[0], y - wo[1], z - wo[2]);
  } else if (g->body) {
    dBodySetPosition(g->body, x, y, z);
  } else {
    g->pos[0] = x; g->pos[1] = y; g->pos[2] = z;
    geom_moved(g);
  }
}
void dGeomSetRotation(dGeomID g, const dMatrix3 R) {
  if (g->has_offset) {
    dReal bpos[3], bR[12];
    body_for_final(g, geom_pos(g), R, bpos, bR);
    dBodySetRotation(g->body, bR);
    dBodySetPosition(g->body, bpos[0], bpos[1], bpos[2]);
  } else if (g->body) {
    dBodySetRotation(g->body, R);
  } else {
    for (int k = 0; k < 12; ++k) g->R[k] = R[k];
    geom_moved(g);
  }
}
void dGeomSetQuaternion(dGeomID g, const dQuaternion q) {
  if (g->has_offset) {
    dReal fR[12], bpos[3], bR[12];
    dRfromQ(fR, q);
    body_for_final(g, geom_pos(g), fR, bpos, bR);
    dBodySetRotation(g->body, bR);
    dBodySetPosition(g->body, bpos[0], bpos[1], bpos[2]);
  }
  // ODE 0.12 tests the body here with a plain `if`, so an offset geom's body
  // then takes the quaternion itself as well (collision_kernel.cpp:630-633)
  if (g->body) {
    dBodySetQuaternion(g->body, q);
  } else {
    dRfromQ(g->R, q);
    geom_moved(g);
  }
}
const dReal* dGeomGetPosition(dGeomID g) { return geom_pos(g); }
const dReal* dGeomGetRotation(dGeomID g) { return geom_R(g); }
void dGeomCopyPosition(dGeomID g, dVector3 pos) {   // :648-657
  const dReal* p = geom_pos(g);
  for (int k = 0; k < 3; ++k) pos[k] = p[k];
}
void dGeomCopyRotation(dGeomID g, dMatrix3 R) {   // :669-685, the pads left alone
  const dReal* s = geom_R(g);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[r * 4 + c] = s[r * 4 + c];
}
void dGeomGetQuaternion(dGeomID g, dQuaternion q) {   // :687-703
  if (g->body && !g->has_offset) {
    for (int k = 0; k < 4; ++k) q[k] = g->body->q[k];
  } else {
    dQfromR(q, geom_R(g));
  }
}

// Each class's computeAABB: sphere.cpp:59-67, box.cpp:60-77,
// capsule.cpp:60-74, cylinder.cpp:59-76, plane.cpp:80-107, ray.cpp:56-89,
// heightfield.cpp:475-600, and a space's union of its geoms'
// (collision_space.cpp:105-126)
static void recompute_aabb(dxGeom* g);
static void compute_aabb(dxGeom* g, dReal* aabb) {
  const float inf = INFINITY;
  if (const dGeomClass* uc = user_class_of(g)) {
    uc->aabb(g, aabb);
    return;
  }
  if (g->type == dGeomTransformClass) {
    // dxGeomTransform::computeAABB (collision_transform.cpp:78-92): the
    // wrapped geom's box at the carried pose, written into the wrapped geom's
    // box as well (its cached box flag untouched), as the reference does
    if (!g->tobj) {
      for (int k = 0; k < 6; ++k) aabb[k] = 0;
      return;
    }
    transform_final(g);
    dxGeom* o = g->tobj;
    o->ovr_pos = g->tpos;
    o->ovr_R = g->tR;
    compute_aabb(o, o->aabb);
    o->ovr_pos = o->ovr_R = nullptr;
    for (int k = 0; k < 6; ++k) aabb[k] = o->aabb[k];
    return;
  }
  if (is_space(g)) {
    const auto* sp = static_cast<const dxSpace*>(g);
    if (sp->qt || sp->sap) {   // these keep the infinite box they start with (quadtree :387-391, SAP :265-271)
      for (int k = 0; k < 6; ++k) aabb[k] = (k & 1) ? inf : -inf;
      return;
    }
    if (!sp->first) {
      for (int k = 0; k < 6; ++k) aabb[k] = 0;
      return;
    }
    for (int k = 0; k < 6; ++k) aabb[k] = (k & 1) ? -inf : inf;
    for (dxGeom* c = sp->first; c; c = c->next) {
      recompute_aabb(c);
      for (int k = 0; k < 6; k += 2) if (c->aabb[k] < aabb[k]) aabb[k] = c->aabb[k];
      for (int k = 1; k < 6; k += 2) if (c->aabb[k] > aabb[k]) aabb[k] = c->aabb[k];
    }
    return;
  }
  if (g->type == dPlaneClass) {
    const dReal p[4] = {(dReal)g->p[0], (dReal)g->p[1], (dReal)g->p[2], (dReal)g->p[3]};
    for (int k = 0; k < 6; ++k) aabb[k] = (k & 1) ? inf : -inf;
    if (p[1] == 0 && p[2] == 0) {
      aabb[0] = p[0] > 0 ? -inf : -p[3];
      aabb[1] = p[0] > 0 ? p[3] : inf;
    } else if (p[0] == 0 && p[2] == 0) {
      aabb[2] = p[1] > 0 ? -inf : -p[3];
      aabb[3] = p[1] > 0 ? p[3] : inf;
    } else if (p[0] == 0 && p[1] == 0) {
      aabb[4] = p[2] > 0 ? -inf : -p[3];
      aabb[5] = p[2] > 0 ? p[3] : inf;
    }
    return;
  }
  if (g->type == dHeightfieldClass) {
    const dxHeightfieldData* d = g->hf;
    if (!d) { for (int k = 0; k < 6; ++k) aabb[k] = 0; return; }
    const float hw = (dReal)d->width / (dReal)2, hd = (dReal)d->depth / (dReal)2;
    if (d->wrap) {
      for (int k = 0; k < 6; ++k) aabb[k] = (k & 1) ? inf : -inf;
      if (!g->placeable) { aabb[2] = d->hmin; aabb[3] = d->hmax; }
      return;
    }
    if (!g->placeable) {
      aabb[0] = -hw; aabb[1] = hw;
      aabb[2] = d->hmin; aabb[3] = d->hmax;
      aabb[4] = -hd; aabb[5] = hd;
      return;
    }
    const dReal* pos = geom_pos(g);
    const dReal* R = geom_R(g);
    dReal dx[6], dy[6], dz[6];
    for (int i = 0; i < 3; ++i) {
      const dReal ry = R[i * 4 + 1];
      // an infinite bound times a zero entry counts as 0, not NaN
      dy[i] = d->hmin != -inf ? ry * d->hmin : (ry ? ry * -inf : 0.f);
      dy[i + 3] = d->hmax != inf ? ry * d->hmax : (ry ? ry * inf : 0.f);
      dx[i] = R[i * 4 + 0] * -hw;
      dx[i + 3] = R[i * 4 + 0] * hw;
      dz[i] = R[i * 4 + 2] * -hd;
      dz[i + 3] = R[i * 4 + 2] * hd;
    }
    for (int i = 0; i < 3; ++i) {
      const dReal lo = std::min(std::min(std::min(dx[i], dx[i + 3]), std::min(dy[i], dy[i + 3])),
                                std::min(dz[i], dz[i + 3]));
      const dReal hi = std::max(std::max(std::max(dx[i], dx[i + 3]), std::max(dy[i], dy[i + 3])),
                                std::max(dz[i], dz[i + 3]));
      aabb[2 * i] = pos[i] + lo;
      aabb[2 * i + 1] = pos[i] + hi;
    }
    return;
  }
  const dReal* pos = geom_pos(g);
  const dReal* R = geom_R(g);
  const dReal a = (dReal)g->p[0], b = (dReal)g->p[1], c = (dReal)g->p[2];
  dReal ext[3];
  switch (g->type) {
    case dSphereClass:
      for (int i = 0; i < 3; ++i) ext[i] = a;
      break;
    case dBoxClass:
      for (int i = 0; i < 3; ++i)
        ext[i] = (dReal)0.5 * (std::fabs(R[i * 4 + 0] * a) + std::fabs(R[i * 4 + 1] * b) + std::fabs(R[i * 4 + 2] * c));
      break;
    case dCapsuleClass:
      for (int i = 0; i < 3; ++i) ext[i] = std::fabs(R[i * 4 + 2] * b) * (dReal)0.5 + a;
      break;
    case dCylinderClass:
      for (int i = 0; i < 3; ++i)
        ext[i] = std::fabs(R[i * 4 + 0] * a) + std::fabs(R[i * 4 + 1] * a) + (dReal)0.5 * std::fabs(R[i * 4 + 2] * b);
      break;
    case dRayClass:
      for (int i = 0; i < 3; ++i) {
        const dReal e = pos[i] + R[i * 4 + 2] * a;
        aabb[2 * i] = pos[i] < e ? pos[i] : e;
        aabb[2 * i + 1] = pos[i] < e ? e : pos[i];
      }
      return;
    default:
      for (int k = 0; k < 6; ++k) aabb[k] = 0;
      return;
  }
  for (int i = 0; i < 3; ++i) {
    aabb[2 * i] = pos[i] - ext[i];
    aabb[2 * i + 1] = pos[i] + ext[i];
  }
}
// dxGeom::recomputeAABB (collision_kernel.h:151-157): the box is cached until
// the geom moves
static void recompute_aabb(dxGeom* g) {
  if (!g->aabb_bad) return;
  compute_aabb(g, g->aabb);
  g->aabb_bad = 0;
}
void dGeomGetAABB(dGeomID g, dReal aabb[6]) {   // collision_kernel.cpp:705-711
  recompute_aabb(g);
  for (int k = 0; k < 6; ++k) aabb[k] = g->aabb[k];
}
// collision_kernel.cpp:714-726
// dClosestLineSegmentPoints (collision_util.cpp:109-209)
void dClosestLineSegmentPoints(const dVector3 a1, const dVector3 a2, const dVector3 b1, const dVector3 b2,
                               dVector3 cp1, dVector3 cp2) {
  og::closest_segment_points_host(a1, a2, b1, b2, cp1, cp2);
}
// dBoxBox (box.cpp:331-713): the box-box collider itself, returning the
// normal, the deepest penetration and the contact code with its contacts'
// positions and depths (at most 8; the caller fills the rest of each record)
int dBoxBox(const dVector3 p1, const dMatrix3 R1, const dVector3 side1, const dVector3 p2, const dMatrix3 R2,
            const dVector3 side2, dVector3 normal, dReal* depth, int* return_code, int flags, dContactGeom* contact,
            int skip) {
  if ((flags & 0xffff) == 0) return 0;
  unsigned f = (unsigned)flags;
  if ((f & 0xffff) > 8) f = (f & ~0xffffu) | 8u;
  og::Contact out[8];
  const int n = og::box_box_host(p1, R1, side1, p2, R2, side2, normal, depth, return_code, f, out);
  for (int i = 0; i < n; ++i) {
    dContactGeom* c = (dContactGeom*)((char*)contact + (size_t)i * skip);
    for (int k = 0; k < 3; ++k) c->pos[k] = out[i].pos[k];
    c->depth = out[i].depth;
  }
  return n;
}
// dBoxTouchesBox (collision_util.cpp:388-449): the fifteen separating axes
// of two boxes (the three faces of each, the nine edge pairs) after
// Gottschalk, Lin and Manocha's OBB tree test, in box 1's frame, with
// R = R1' R2 and Q = |R|
int dBoxTouchesBox(const dVector3 p1, const dMatrix3 R1, const dVector3 side1, const dVector3 p2,
                   const dMatrix3 R2, const dVector3 side2) {
  const dReal p[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
  dReal pp[3], A[3], B[3], R[3][3], Q[3][3];
  for (int i = 0; i < 3; ++i) {
    pp[i] = R1[i] * p[0] + R1[4 + i] * p[1] + R1[8 + i] * p[2];
    A[i] = side1[i] * (dReal)0.5;
    B[i] = side2[i] * (dReal)0.5;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      R[i][j] = R1[i] * R2[j] + R1[4 + i] * R2[4 + j] + R1[8 + i] * R2[8 + j];
      Q[i][j] = std::fabs(R[i][j]);
    }
  for (int i = 0; i < 3; ++i)   // box 1's faces
    if (std::fabs(pp[i]) > A[i] + B[0] * Q[i][0] + B[1] * Q[i][1] + B[2] * Q[i][2]) return 0;
  for (int j = 0; j < 3; ++j) {   // box 2's faces
    const dReal d = R2[j] * p[0] + R2[4 + j] * p[1] + R2[8 + j] * p[2];
    if (std::fabs(d) > A[0] * Q[0][j] + A[1] * Q[1][j] + A[2] * Q[2][j] + B[j]) return 0;
  }
  for (int i = 0; i < 3; ++i) {   // edge i of box 1 against edge j of box 2
    const int a = (i + 1) % 3, b = (i + 2) % 3, m = a < b ? a : b, n = a < b ? b : a;
    for (int j = 0; j < 3; ++j) {
      const int k = j == 0 ? 1 : 0, l = j == 2 ? 1 : 2;
      if (std::fabs(pp[b] * R[a][j] - pp[a] * R[b][j]) > A[m] * Q[n][j] + A[n] * Q[m][j] + B[k] * Q[i][l] + B[l] * Q[i][k])
        return 0;
    }
  }
  return 1;
}
void dInfiniteAABB(dGeomID, dReal aabb[6]) {   // collision_util.cpp:457-465
  for (int k = 0; k < 6; ++k) aabb[k] = (k & 1) ? INFINITY : -INFINITY;
}
// dGeomLowLevelControl (collision_kernel.cpp:877-889): only trimeshes take
// controls in ODE 0.12; every class here answers none
int dGeomLowLevelControl(dGeomID g, int, int, void*, int* dataSize) {
  if (!g || !dataSize) return 0;
  *dataSize = 0;
  return 0;
}
int dGeomIsSpace(dGeomID g) { return is_space(g) ? 1 : 0; }
dSpaceID dGeomGetSpace(dGeomID g) { return g->space; }
int dGeomGetClass(dGeomID g) { return g->type; }
// Category / collide bits and the enabled flag (collision_kernel.cpp:735-782)
// steer a space's pair search only; dCollide reads none of them.
void dGeomSetCategoryBits(dGeomID g, unsigned long bits) { g->category_bits = bits; }
void dGeomSetCollideBits(dGeomID g, unsigned long bits) { g->collide_bits = bits; }
unsigned long dGeomGetCategoryBits(dGeomID g) { return g->category_bits; }
unsigned long dGeomGetCollideBits(dGeomID g) { return g->collide_bits; }
void dGeomEnable(dGeomID g) { g->enabled = 1; }
void dGeomDisable(dGeomID g) { g->enabled = 0; }
int dGeomIsEnabled(dGeomID g) { return g->enabled != 0; }
// Geom-frame points and vectors (collision_kernel.cpp:784-874); a geom
// without a pose passes them through
void dGeomGetRelPointPos(dGeomID g, dReal px, dReal py, dReal pz, dVector3 result) {
  if (!geom_placeable(g)) { result[0] = px; result[1] = py; result[2] = pz; return; }
  const dReal* pos = geom_pos(g);
  const dReal v[3] = {px, py, pz};
  dReal a[3];
  mul0_331(a, geom_R(g), v);
  for (int k = 0; k < 3; ++k) result[k] = a[k] + pos[k];
}
void dGeomGetPosRelPoint(dGeomID g, dReal px, dReal py, dReal pz, dVector3 result) {
  if (!geom_placeable(g)) { result[0] = px; result[1] = py; result[2] = pz; return; }
  const dReal* pos = geom_pos(g);
  const dReal v[3] = {px - pos[0], py - pos[1], pz - pos[2]};
  mul1_331(result, geom_R(g), v);
}
void dGeomVectorToWorld(dGeomID g, dReal px, dReal py, dReal pz, dVector3 result) {
  if (!geom_placeable(g)) { result[0] = px; result[1] = py; result[2] = pz; return; }
  const dReal v[3] = {px, py, pz};
  mul0_331(result, geom_R(g), v);
}
void dGeomVectorFromWorld(dGeomID g, dReal px, dReal py, dReal pz, dVector3 result) {
  if (!geom_placeable(g)) { result[0] = px; result[1] = py; result[2] = pz; return; }
  const dReal v[3] = {px, py, pz};
  mul1_331(result, geom_R(g), v);
}

// Offsets from the body (collision_kernel.cpp:1036-1250). Setting one on a
// geom without a body does nothing.
void dGeomSetOffsetPosition(dGeomID g, dReal x, dReal y, dReal z) {
  if (!geom_make_offset(g)) return;
  g->opos[0] = x; g->opos[1] = y; g->opos[2] = z;
  geom_moved(g);
}
void dGeomSetOffsetRotation(dGeomID g, const dMatrix3 R) {
  if (!geom_make_offset(g)) return;
  for (int k = 0; k < 12; ++k) g->oR[k] = R[k];
  geom_moved(g);
}
void dGeomSetOffsetQuaternion(dGeomID g, const dQuaternion q) {
  if (!geom_make_offset(g)) return;
  dRfromQ(g->oR, q);
  geom_moved(g);
}
void dGeomSetOffsetWorldPosition(dGeomID g, dReal x, dReal y, dReal z) {
  if (!geom_make_offset(g)) return;
  dBodyGetPosRelPoint(g->body, x, y, z, g->opos);
  geom_moved(g);
}
void dGeomSetOffsetWorldRotation(dGeomID g, const dMatrix3 R) {
  if (!geom_make_offset(g)) return;
  dReal fpos[3];
  const dReal* p = geom_pos(g);
  for (int k = 0; k < 3; ++k) fpos[k] = p[k];
  offset_for_final(g, fpos, R);
  geom_moved(g);
}
void dGeomSetOffsetWorldQuaternion(dGeomID g, const dQuaternion q) {
  if (!geom_make_offset(g)) return;
  dReal fpos[3], fR[12];
  const dReal* p = geom_pos(g);
  for (int k = 0; k < 3; ++k) fpos[k] = p[k];
  dRfromQ(fR, q);
  offset_for_final(g, fpos, fR);
  geom_moved(g);
}
void dGeomClearOffset(dGeomID g) {
  if (!g->has_offset) return;
  g->has_offset = 0;
  geom_moved(g);
}
int dGeomIsOffset(dGeomID g) { return g->has_offset ? 1 : 0; }
static const dReal kZeroOffsetPos[4] = {0, 0, 0, 0};
static const dReal kZeroOffsetR[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
const dReal* dGeomGetOffsetPosition(dGeomID g) { return g->has_offset ? g->opos : kZeroOffsetPos; }
void dGeomCopyOffsetPosition(dGeomID g, dVector3 pos) {
  const dReal* p = dGeomGetOffsetPosition(g);
  for (int k = 0; k < 3; ++k) pos[k] = p[k];
}
const dReal* dGeomGetOffsetRotation(dGeomID g) { return g->has_offset ? g->oR : kZeroOffsetR; }
void dGeomCopyOffsetRotation(dGeomID g, dMatrix3 R) {
  const dReal* s = dGeomGetOffsetRotation(g);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[r * 4 + c] = s[r * 4 + c];
}
void dGeomGetOffsetQuaternion(dGeomID g, dQuaternion q) {
  if (g->has_offset) {
    dQfromR(q, g->oR);
  } else {
    q[0] = 1; q[1] = q[2] = q[3] = 0;
  }
}

// ---------------------------------------------------------------- class parameters
// Setters of sphere.cpp:76-84, box.cpp:86-96, plane.cpp:117-127,
// capsule.cpp:83-92; the point depths of sphere.cpp:95-105, box.cpp:109-173,
// plane.cpp:141-146, capsule.cpp:104-126, in dReal arithmetic.
dReal dGeomSphereGetRadius(dGeomID g) { return (dReal)g->p[0]; }
void dGeomSphereSetRadius(dGeomID g, dReal radius) {
  if (!g || g->type != dSphereClass) return;
  g->p[0] = radius;
  g->zero_sized = radius == 0;
  geom_moved(g);
}
dReal dGeomSpherePointDepth(dGeomID g, dReal x, dReal y, dReal z) {
  const dReal* pos = geom_pos(g);
  return (dReal)g->p[0] - std::sqrt((x - pos[0]) * (x - pos[0]) + (y - pos[1]) * (y - pos[1]) +
                                    (z - pos[2]) * (z - pos[2]));
}
void dGeomBoxGetLengths(dGeomID g, dVector3 r) { for (int k = 0; k < 3; ++k) r[k] = (dReal)g->p[k]; }
void dGeomBoxSetLengths(dGeomID g, dReal lx, dReal ly, dReal lz) {
  if (!g || g->type != dBoxClass) return;
  g->p[0] = lx; g->p[1] = ly; g->p[2] = lz;
  g->zero_sized = lx == 0 || ly == 0 || lz == 0;
  geom_moved(g);
}
dReal dGeomBoxPointDepth(dGeomID g, dReal x, dReal y, dReal z) {
  const dReal* pos = geom_pos(g);
  const dReal p[3] = {x - pos[0], y - pos[1], z - pos[2]};
  dReal q[3], dist[6];
  mul1_331(q, geom_R(g), p);
  bool inside = true;
  for (int i = 0; i < 3; ++i) {
    const dReal side = (dReal)g->p[i] * (dReal)0.5;
    dist[i] = side - q[i];
    dist[i + 3] = side + q[i];
    if (dist[i] < 0 || dist[i + 3] < 0) inside = false;
  }
  if (inside) {   // the nearest face
    dReal m = (dReal)4294967295.0;
    for (int i = 0; i < 6; ++i) if (dist[i] < m) m = dist[i];
    return m;
  }
  dReal m = 0;   // outside: minus the largest face distance
  for (int i = 0; i < 6; ++i) if (dist[i] > m) m = dist[i];
  return -m;
}
void dGeomPlaneGetParams(dGeomID g, dVector4 r) { for (int k = 0; k < 4; ++k) r[k] = (dReal)g->p[k]; }
void dGeomPlaneSetParams(dGeomID g, dReal a, dReal b, dReal c, dReal d) {
  if (!g || g->type != dPlaneClass) return;
  plane_params(g->p, a, b, c, d);
  geom_moved(g);
}
dReal dGeomPlanePointDepth(dGeomID g, dReal x, dReal y, dReal z) {
  const dReal p[4] = {(dReal)g->p[0], (dReal)g->p[1], (dReal)g->p[2], (dReal)g->p[3]};
  return p[3] - p[0] * x - p[1] * y - p[2] * z;
}
void dGeomCapsuleGetParams(dGeomID g, dReal* r, dReal* l) { *r = (dReal)g->p[0]; *l = (dReal)g->p[1]; }
void dGeomCapsuleSetParams(dGeomID g, dReal radius, dReal length) {
  if (!g || g->type != dCapsuleClass) return;
  g->p[0] = radius; g->p[1] = length;
  g->zero_sized = radius == 0;
  geom_moved(g);
}
dReal dGeomCapsulePointDepth(dGeomID g, dReal x, dReal y, dReal z) {
  const dReal* R = geom_R(g);
  const dReal* pos = geom_pos(g);
  const dReal a[3] = {x - pos[0], y - pos[1], z - pos[2]};
  dReal beta = a[0] * R[2] + a[1] * R[6] + a[2] * R[10];
  const dReal lz2 = (dReal)g->p[1] * (dReal)0.5;
  if (beta < -lz2) beta = -lz2;
  else if (beta > lz2) beta = lz2;
  const dReal c[3] = {pos[0] + beta * R[2], pos[1] + beta * R[6], pos[2] + beta * R[10]};
  return (dReal)g->p[0] - std::sqrt((x - c[0]) * (x - c[0]) + (y - c[1]) * (y - c[1]) + (z - c[2]) * (z - c[2]));
}

// User geoms (collision_kernel.cpp:900-938, :993-1012): placeable, in no
// space, with a zeroed block of the class's size; the class gives the box, an
// optional box test for space pairs and a destructor
dGeomID dCreateGeom(int classnum) {
  if (!is_user_class(classnum)) return nullptr;
  const double p[4] = {0, 0, 0, 0};
  dGeomID g = new_geom(nullptr, classnum, p);
  const int bytes = g_user_classes[classnum - kFirstUserClass].bytes;
  g->class_data = std::calloc(1, bytes > 0 ? (size_t)bytes : 1);
  return g;
}
void* dGeomGetClassData(dGeomID g) { return g && is_user_class(g->type) ? g->class_data : nullptr; }
static const dGeomClass* user_class_of(const dxGeom* g) {
  return is_user_class(g->type) ? &g_user_classes[g->type - kFirstUserClass] : nullptr;
}

// Geom transforms (collision_transform.cpp:153-209): a placeable geom that
// carries another one (not in a space, not on a body) at its own pose
dGeomID dCreateGeomTransform(dSpaceID space) {
  const double p[4] = {0, 0, 0, 0};
  return new_geom(space, dGeomTransformClass, p);
}
void dGeomTransformSetGeom(dGeomID g, dGeomID obj) {
  if (!g || g->type != dGeomTransformClass) return;
  if (g->tobj && g->tcleanup) dGeomDestroy(g->tobj);
  g->tobj = obj;
}
dGeomID dGeomTransformGetGeom(dGeomID g) { return g && g->type == dGeomTransformClass ? g->tobj : nullptr; }
void dGeomTransformSetCleanup(dGeomID g, int mode) { if (g && g->type == dGeomTransformClass) g->tcleanup = mode; }
int dGeomTransformGetCleanup(dGeomID g) { return g && g->type == dGeomTransformClass ? g->tcleanup : 0; }
void dGeomTransformSetInfo(dGeomID g, int mode) { if (g && g->type == dGeomTransformClass) g->tinfo = mode; }
int dGeomTransformGetInfo(dGeomID g) { return g && g->type == dGeomTransformClass ? g->tinfo : 0; }

// ---------------------------------------------------------------- spaces (API)
// Simple and hash spaces (collision_space.cpp:210-604) on the host: they only
// enumerate candidate pairs for the caller's near-callback, which calls
// dCollide. Sweep-and-prune and quadtree spaces are not built.
static dSpaceID new_space(dSpaceID parent, int type) {
  auto* sp = new dxSpace();
  std::memset(static_cast<dxGeom*>(sp), 0, sizeof(dxGeom));
  sp->first = nullptr;
  sp->count = 0;
  sp->cleanup = 1;
  sp->sublevel = 0;
  sp->manual_cleanup = 0;
  sp->minlevel = -3;   // dxHashSpace::dxHashSpace (collision_space.cpp:385-390)
  sp->maxlevel = 10;
  init_geom(sp, parent, type);
  return sp;
}
static bool geom_enabled(const dxGeom* g) { return g->enabled && !g->zero_sized; }   // GEOM_ENABLED
// collideAABBs (collision_space_internal.h:48-82)
static void collide_aabbs(dxGeom* g1, dxGeom* g2, void* data, dNearCallback* cb) {
  if (g1->body == g2->body && g1->body) return;
  if (((g1->category_bits & g2->collide_bits) || (g2->category_bits & g1->collide_bits)) == 0) return;
  const dReal* a = g1->aabb;
  const dReal* b = g2->aabb;
  if (a[0] > b[1] || a[1] < b[0] || a[2] > b[3] || a[3] < b[2] || a[4] > b[5] || a[5] < b[4]) return;
  // a user class may prove the boxes apart (dxUserGeom::AABBTest)
  const dGeomClass* u1 = user_class_of(g1);
  const dGeomClass* u2 = user_class_of(g2);
  if (u1 && u1->aabb_test && u1->aabb_test(g1, g2, g2->aabb) == 0) return;
  if (u2 && u2->aabb_test && u2->aabb_test(g2, g1, g1->aabb) == 0) return;
  cb(data, g1, g2);
}
// cleanGeoms (collision_space.cpp:229-242, :390-402): boxes of the dirty
// prefix, nested spaces first
static void space_clean(dxSpace* sp) {
  if (sp->sap) {   // dxSAPSpace::cleanGeoms (:394-423): the dirty list onto the clean one
    SapSpace& S = *sp->sap;
    for (dxGeom* g : S.dirty) {
      if (is_space(g)) space_clean(static_cast<dxSpace*>(g));
      recompute_aabb(g);
      g->dirty = g->aabb_bad = 0;
      g->sap_dirty = -1;
      g->sap_clean = (int)S.geoms.size();
      S.geoms.push_back(g);
    }
    S.dirty.clear();
    return;
  }
  if (sp->qt) {   // dxQuadTreeSpace::cleanGeoms (:542-559): boxes, then each geom to its block
    QuadTree& q = *sp->qt;
    for (size_t i = 0; i < q.dirty.size(); ++i) {
      dxGeom* g = q.dirty[i];
      if (is_space(g)) space_clean(static_cast<dxSpace*>(g));
      recompute_aabb(g);
      g->dirty = g->aabb_bad = 0;
      const int nb = quad_block(q, g->qblock, g->aabb);
      if (nb != g->qblock) {
        quad_del(q, g);
        quad_add(q, nb, g);
      }
    }
    q.dirty.clear();
    return;
  }
  for (dxGeom* g = sp->first; g && g->dirty; g = g->next) {
    if (is_space(g)) space_clean(static_cast<dxSpace*>(g));
    recompute_aabb(g);
    g->dirty = g->aabb_bad = 0;
  }
}
// dxSimpleSpace::collide (collision_space.cpp:245-264): every pair in list order
static void simple_collide(dxSpace* sp, void* data, dNearCallback* cb) {
  space_clean(sp);
  for (dxGeom* g1 = sp->first; g1; g1 = g1->next) {
    if (!geom_enabled(g1)) continue;
    for (dxGeom* g2 = g1->next; g2; g2 = g2->next)
      if (geom_enabled(g2)) collide_aabbs(g1, g2, data, cb);
  }
}
// collide2 of both space kinds (:267-283, :589-604): the geom against each member
static void quad_collide2(dxSpace* sp, void* data, dxGeom* geom, dNearCallback* cb);
static void space_collide2(dxSpace* sp, void* data, dxGeom* geom, dNearCallback* cb) {
  if (sp->qt) {
    quad_collide2(sp, data, geom, cb);
    return;
  }
  if (sp->sap) {   // dxSAPSpace::collide2 (:498-519): every clean member, boxes tested
    space_clean(sp);
    recompute_aabb(geom);
    for (size_t i = 0; i < sp->sap->geoms.size(); ++i) {
      dxGeom* g = sp->sap->geoms[i];
      if (geom_enabled(g)) collide_aabbs(g, geom, data, cb);
    }
    return;
  }
  space_clean(sp);
  recompute_aabb(geom);
  for (dxGeom* g = sp->first; g; g = g->next)
    if (geom_enabled(g)) collide_aabbs(g, geom, data, cb);
}
// findLevel (collision_space.cpp:325-347): the smallest cell level whose cell
// is at least the box's largest side; boxes with an infinite side get none
static int hash_level(const dReal* b) {
  if (b[0] <= -INFINITY || b[1] >= INFINITY || b[2] <= -INFINITY || b[3] >= INFINITY || b[4] <= -INFINITY ||
      b[5] >= INFINITY)
    return INT_MAX;
  dReal q = b[1] - b[0], q2 = b[3] - b[2];
  if (q2 > q) q = q2;
  q2 = b[5] - b[4];
  if (q2 > q) q = q2;
  int level = 0;
  std::frexp(q, &level);
  return level;
}
// getVirtualAddress (collision_space.cpp:354-357), int arithmetic widened to
// unsigned long as there
static unsigned long hash_cell(int level, int x, int y, int z) {
  const int v = (int)((unsigned)level * 1000u + (unsigned)x * 100u + (unsigned)y * 10u + (unsigned)z);
  return (unsigned long)(long)v;
}
// dxHashSpace::collide (collision_space.cpp:405-586): boxes binned into cells
// of 2^level per level, cell buckets chained newest first, each pair tested
// once through an n x n bit table, then the boxes too large for any level
// against all the others and among themselves
static void hash_collide(dxSpace* sp, void* data, dNearCallback* cb) {
  static const long kPrime[31] = {1L, 2L, 3L, 7L, 13L, 31L, 61L, 127L, 251L, 509L, 1021L, 2039L, 4093L,
                                  8191L, 16381L, 32749L, 65521L, 131071L, 262139L, 524287L, 1048573L,
                                  2097143L, 4194301L, 8388593L, 16777213L, 33554393L, 67108859L,
                                  134217689L, 268435399L, 536870909L, 1073741789L};   // largest prime < 2^i
  if (sp->count < 2) return;
  space_clean(sp);
  struct Box { int next, level, db[6], index; dxGeom* g; };
  std::vector<Box> box;
  box.reserve(sp->count);
  int first = -1, big = -1, n = 0, maxlevel = sp->minlevel - 1;
  for (dxGeom* g = sp->first; g; g = g->next) {
    if (!geom_enabled(g)) continue;
    Box b{};
    b.g = g;
    int level = hash_level(g->aabb);
    if (level < sp->minlevel) level = sp->minlevel;
    const int id = (int)box.size();
    if (level <= sp->maxlevel) {
      b.next = first;
      first = id;
      b.level = level;
      if (level > maxlevel) maxlevel = level;
      const dReal cell = (dReal)std::ldexp(1.0, level);
      for (int i = 0; i < 6; ++i) b.db[i] = (int)std::floor(g->aabb[i] / cell);
      b.index = n++;
    } else {
      b.next = big;
      big = id;
    }
    box.push_back(b);
  }
  const int rowsize = (n + 7) >> 3;
  std::vector<unsigned char> tested((size_t)n * rowsize, 0);
  int pi = 0;
  while (pi < 31 && kPrime[pi] < 8L * n) ++pi;
  if (pi >= 31) pi = 30;
  const unsigned long sz = (unsigned long)kPrime[pi];
  struct Node { int next, x, y, z, box; };
  std::vector<int> table(sz, -1);
  std::vector<Node> node;
  for (int a = first; a >= 0; a = box[a].next) {
    const Box& b = box[a];
    for (int x = b.db[0]; x <= b.db[1]; ++x)
      for (int y = b.db[2]; y <= b.db[3]; ++y)
        for (int z = b.db[4]; z <= b.db[5]; ++z) {
          const unsigned long h = hash_cell(b.level, x, y, z) % sz;
          node.push_back({table[h], x, y, z, a});
          table[h] = (int)node.size() - 1;
        }
  }
  for (int a = first; a >= 0; a = box[a].next) {
    int db[6];
    for (int i = 0; i < 6; ++i) db[i] = box[a].db[i];
    for (int level = box[a].level; level <= maxlevel; ++level) {
      for (int x = db[0]; x <= db[1]; ++x)
        for (int y = db[2]; y <= db[3]; ++y)
          for (int z = db[4]; z <= db[5]; ++z) {
            const unsigned long h = hash_cell(level, x, y, z) % sz;
            for (int k = table[h]; k >= 0; k = node[k].next) {
              const Node& nd = node[k];
              if (nd.box == a) continue;
              const Box& o = box[nd.box];
              if (o.level != level || nd.x != x || nd.y != y || nd.z != z) continue;
              const int ia = box[a].index, io = o.index;
              const size_t bit = ia <= io ? (size_t)ia * rowsize + (io >> 3) : (size_t)io * rowsize + (ia >> 3);
              const unsigned char mask = (unsigned char)(1u << ((ia <= io ? io : ia) & 7));
              if ((tested[bit] & mask) == 0) collide_aabbs(box[a].g, o.g, data, cb);
              tested[bit] |= mask;
            }
          }
      for (int i = 0; i < 6; ++i) db[i] >>= 1;   // the cell one level up
    }
  }
  for (int a = first; a >= 0; a = box[a].next)
    for (int b = big; b >= 0; b = box[b].next) collide_aabbs(box[a].g, box[b].g, data, cb);
  for (int a = big; a >= 0; a = box[a].next)
    for (int b = box[a].next; b >= 0; b = box[b].next) collide_aabbs(box[a].g, box[b].g, data, cb);
}
// Block::Collide (collision_quadtreespace.cpp:177-238): each enabled geom of
// a block against the later ones in its list and, through the children whose
// box its box reaches (every child holding one geom is visited), against the
// geoms below; then the children holding two or more geoms in turn
static void quad_collide_geom(const QuadTree& q, int b, dxGeom* g1, dxGeom* g2, void* data, dNearCallback* cb) {
  for (; g2; g2 = g2->next)
    if (geom_enabled(g2)) collide_aabbs(g1, g2, data, cb);
  const int c = q.blocks[b].children;
  if (c < 0) return;
  for (int i = 0; i < 4; ++i) {
    const QuadBlock& ch = q.blocks[c + i];
    if (ch.count == 0) continue;
    if (ch.count != 1 && (g1->aabb[0] >= ch.maxx || g1->aabb[1] < ch.minx || g1->aabb[2] >= ch.maxy ||
                          g1->aabb[3] < ch.miny))
      continue;
    quad_collide_geom(q, c + i, g1, ch.first, data, cb);
  }
}
static void quad_collide_block(const QuadTree& q, int b, void* data, dNearCallback* cb) {
  for (dxGeom* g = q.blocks[b].first; g; g = g->next)
    if (geom_enabled(g)) quad_collide_geom(q, b, g, g->next, data, cb);
  const int c = q.blocks[b].children;
  if (c < 0) return;
  for (int i = 0; i < 4; ++i)
    if (q.blocks[c + i].count > 1) quad_collide_block(q, c + i, data, cb);
}
const uint32_t* RadixSorter::sort(const float* keys, uint32_t nb) {
  if (nb != used) {   // ReallocateRanksIfNecessary
    if (nb > size) {
      buf.assign(2 * (size_t)nb, 0);
      size = nb;
      primary = 0;
    }
    valid = false;
    used = nb;
  }
  uint32_t hist[4][256] = {};
  auto byte_of = [&](uint32_t i, int pass) {
    uint32_t v;
    std::memcpy(&v, keys + i, 4);
    return (v >> (8 * pass)) & 0xffu;
  };
  // histograms, and the already-sorted test along the previous order
  bool sorted = true;
  uint32_t k = 0;
  if (!valid) {
    for (; k < nb; ++k) {
      if (k > 0 && keys[k] < keys[k - 1]) { sorted = false; break; }
      for (int pass = 0; pass < 4; ++pass) ++hist[pass][byte_of(k, pass)];
    }
    if (sorted) {
      for (uint32_t i = 0; i < nb; ++i) ranks1()[i] = i;
      return ranks1();
    }
  } else {
    const uint32_t* r = ranks1();
    for (; k < nb; ++k) {
      if (k > 0 && keys[r[k]] < keys[r[k - 1]]) { sorted = false; break; }
      for (int pass = 0; pass < 4; ++pass) ++hist[pass][byte_of(k, pass)];
    }
    if (sorted) return ranks1();
  }
  for (; k < nb; ++k)
    for (int pass = 0; pass < 4; ++pass) ++hist[pass][byte_of(k, pass)];
  uint32_t negatives = 0;
  for (int i = 128; i < 256; ++i) negatives += hist[3][i];
  for (int pass = 0; pass < 4; ++pass) {
    const uint32_t* count = hist[pass];
    const uint32_t unique = byte_of(0, pass);
    const bool perform = count[unique] != nb;
    if (pass != 3) {
      if (!perform) continue;
      uint32_t* out = ranks2();
      uint32_t* link[256];
      link[0] = out;
      for (int i = 1; i < 256; ++i) link[i] = link[i - 1] + count[i - 1];
      if (!valid) {
        for (uint32_t i = 0; i < nb; ++i) *link[byte_of(i, pass)]++ = i;
        valid = true;
      } else {
        const uint32_t* in = ranks1();
        for (uint32_t i = 0; i < nb; ++i) *link[byte_of(in[i], pass)]++ = in[i];
      }
      swap();
    } else if (perform) {
      uint32_t* out = ranks2();
      uint32_t* link[256];
      link[0] = out + negatives;   // positives after the negatives
      for (int i = 1; i < 128; ++i) link[i] = link[i - 1] + count[i - 1];
      link[255] = out;             // negatives in reverse
      for (int i = 0; i < 127; ++i) link[254 - i] = link[255 - i] + count[255 - i];
      for (int i = 128; i < 256; ++i) link[i] += count[i];
      if (!valid) {
        for (uint32_t i = 0; i < nb; ++i) {
          const uint32_t radix = byte_of(i, 3);
          if (radix < 128) *link[radix]++ = i;
          else *(--link[radix]) = i;
        }
        valid = true;
      } else {
        const uint32_t* in = ranks1();
        for (uint32_t i = 0; i < nb; ++i) {
          const uint32_t radix = byte_of(in[i], 3);
          if (radix < 128) *link[radix]++ = in[i];
          else *(--link[radix]) = in[i];
        }
      }
      swap();
    } else if (unique >= 128) {   // all negative: the order reversed
      uint32_t* out = ranks2();
      if (!valid) {
        for (uint32_t i = 0; i < nb; ++i) out[i] = nb - i - 1;
        valid = true;
      } else {
        const uint32_t* in = ranks1();
        for (uint32_t i = 0; i < nb; ++i) out[i] = in[nb - i - 1];
      }
      swap();
    }
  }
  return ranks1();
}
// collideGeomsNoAABBs (collision_sapspace.cpp:234-257): collideAABBs without
// the box overlap test, which the sweep has done
static void sap_collide_pair(dxGeom* g1, dxGeom* g2, void* data, dNearCallback* cb) {
  if (g1->body == g2->body && g1->body) return;
  if (((g1->category_bits & g2->collide_bits) || (g2->category_bits & g1->collide_bits)) == 0) return;
  const dGeomClass* u1 = user_class_of(g1);
  const dGeomClass* u2 = user_class_of(g2);
  if (u1 && u1->aabb_test && u1->aabb_test(g1, g2, g2->aabb) == 0) return;
  if (u2 && u2->aabb_test && u2->aabb_test(g2, g1, g1->aabb) == 0) return;
  cb(data, g1, g2);
}
// dxSAPSpace::collide and BoxPruning (collision_sapspace.cpp:425-496,
// :521-575): enabled geoms split by an infinite upper bound on the first
// axis; the finite ones sorted by their lower bound on it and swept, each
// against the ones that start before it ends, kept when the other two axes
// overlap; then the infinite ones against each other and against the rest
static void sap_collide(dxSpace* sp, void* data, dNearCallback* cb) {
  space_clean(sp);
  SapSpace& S = *sp->sap;
  S.tmp.clear();
  S.tmp_inf.clear();
  for (dxGeom* g : S.geoms) {
    if (!geom_enabled(g)) continue;
    (g->aabb[S.ax0 + 1] == INFINITY ? S.tmp_inf : S.tmp).push_back(g);
  }
  std::vector<std::pair<uint32_t, uint32_t>> overlap;
  const uint32_t n = (uint32_t)S.tmp.size();
  if (n > 0) {
    S.pos.resize(n + 1);
    for (uint32_t i = 0; i < n; ++i) S.pos[i] = (float)S.tmp[i]->aabb[S.ax0];
    S.pos[n] = FLT_MAX;
    const uint32_t count = n + 1;
    const uint32_t* sorted = S.sorter.sort(S.pos.data(), count);
    const uint32_t* last = sorted + count;
    const uint32_t* running = sorted;
    while (running < last && sorted < last) {
      const uint32_t id0 = *sorted++;
      while (S.pos[*running++] < S.pos[id0]) {
      }
      if (running < last) {
        const uint32_t* running2 = running;
        const dReal* a0 = S.tmp[id0]->aabb;
        const dReal max0 = a0[S.ax0 + 1], max1 = a0[S.ax1 + 1], max2 = a0[S.ax2 + 1];
        uint32_t id1;
        while (S.pos[id1 = *running2++] <= max0) {
          const dReal* a1 = S.tmp[id1]->aabb;
          if (max1 >= a1[S.ax1] && a1[S.ax1 + 1] >= a0[S.ax1] && max2 >= a1[S.ax2] && a1[S.ax2 + 1] >= a0[S.ax2])
            overlap.push_back({id0, id1});
        }
      }
    }
  }
  for (const auto& pr : overlap) sap_collide_pair(S.tmp[pr.first], S.tmp[pr.second], data, cb);
  for (size_t m = 0; m < S.tmp_inf.size(); ++m) {
    for (size_t k = m + 1; k < S.tmp_inf.size(); ++k) sap_collide_pair(S.tmp_inf[m], S.tmp_inf[k], data, cb);
    for (dxGeom* g2 : S.tmp) sap_collide_pair(S.tmp_inf[m], g2, data, cb);
  }
}
static void space_collide(dxSpace* sp, void* data, dNearCallback* cb) {
  if (sp->sap) {
    sap_collide(sp, data, cb);
  } else if (sp->qt) {
    space_clean(sp);
    quad_collide_block(*sp->qt, 0, data, cb);
  } else if (sp->type == dHashSpaceClass) {
    hash_collide(sp, data, cb);
  } else {
    simple_collide(sp, data, cb);
  }
}

dSpaceID dSimpleSpaceCreate(dSpaceID space) { return new_space(space, dSimpleSpaceClass); }
dSpaceID dHashSpaceCreate(dSpaceID space) { return new_space(space, dHashSpaceClass); }
// dQuadTreeSpaceCreate (collision_quadtreespace.cpp:362-392, :134-175): the
// root spans center +- extents on x and y, its upper edges nudged up to the
// next float so that they are inside; depth levels of four children each
static void quad_build(QuadTree& q, int b, dReal minx, dReal maxx, dReal miny, dReal maxy, int parent, int depth) {
  q.blocks[b] = {minx, maxx, miny, maxy, nullptr, 0, parent, -1};
  if (depth <= 0) return;
  const int c = (int)q.blocks.size();
  q.blocks[b].children = c;
  q.blocks.resize(q.blocks.size() + 4);
  const dReal ex = (maxx - minx) / 2, ey = (maxy - miny) / 2;
  dReal right_x = minx;
  int k = 0;
  for (int i = 0; i < 2; ++i) {
    const dReal left_x = right_x;
    right_x = i != 1 ? left_x + ex : maxx;
    dReal right_y = miny;
    for (int j = 0; j < 2; ++j) {
      const dReal left_y = right_y;
      right_y = j != 1 ? left_y + ey : maxy;
      quad_build(q, c + k++, left_x, right_x, left_y, right_y, b, depth - 1);
    }
  }
}
// dSweepAndPruneSpaceCreate (collision_sapspace.cpp:210-213, :261-276): the
// sweep axis and the two test axes from the axis order's three 2-bit fields
dSpaceID dSweepAndPruneSpaceCreate(dSpaceID space, int axisorder) {
  auto* S = new SapSpace();
  S->ax0 = (axisorder & 3) << 1;
  S->ax1 = ((axisorder >> 2) & 3) << 1;
  S->ax2 = ((axisorder >> 4) & 3) << 1;
  dSpaceID sp = new_space(nullptr, dSweepAndPruneSpaceClass);
  sp->sap = S;
  if (space) space_add(space, sp);
  return sp;
}
dSpaceID dQuadTreeSpaceCreate(dSpaceID space, const dVector3 Center, const dVector3 Extents, int Depth) {
  auto* q = new QuadTree();
  q->blocks.resize(1);
  quad_build(*q, 0, Center[0] - Extents[0], std::nextafter((dReal)(Center[0] + Extents[0]), (dReal)INFINITY),
             Center[1] - Extents[1], std::nextafter((dReal)(Center[1] + Extents[1]), (dReal)INFINITY), -1,
             Depth < 0 ? 0 : Depth);
  dSpaceID sp = new_space(nullptr, dQuadTreeSpaceClass);
  sp->qt = q;
  if (space) space_add(space, sp);
  return sp;
}
void dHashSpaceSetLevels(dSpaceID space, int minlevel, int maxlevel) {
  if (!space || space->type != dHashSpaceClass || minlevel > maxlevel) return;
  space->minlevel = minlevel;
  space->maxlevel = maxlevel;
}
void dHashSpaceGetLevels(dSpaceID space, int* minlevel, int* maxlevel) {
  if (!space || space->type != dHashSpaceClass) return;
  if (minlevel) *minlevel = space->minlevel;
  if (maxlevel) *maxlevel = space->maxlevel;
}
void dSpaceDestroy(dSpaceID space) { dGeomDestroy(space); }
void dSpaceSetCleanup(dSpaceID space, int mode) { space->cleanup = mode != 0; }
int dSpaceGetCleanup(dSpaceID space) { return space->cleanup; }
void dSpaceSetSublevel(dSpaceID space, int sublevel) { space->sublevel = sublevel; }
int dSpaceGetSublevel(dSpaceID space) { return space->sublevel; }
void dSpaceSetManualCleanup(dSpaceID space, int mode) { space->manual_cleanup = mode; }
int dSpaceGetManualCleanup(dSpaceID space) { return space->manual_cleanup; }
void dSpaceAdd(dSpaceID space, dGeomID g) { space_add(space, g); }
void dSpaceRemove(dSpaceID space, dGeomID g) { space_remove(space, g); }
int dSpaceQuery(dSpaceID space, dGeomID g) { return g && g->space == space ? 1 : 0; }
void dSpaceClean(dSpaceID space) { space_clean(space); }
int dSpaceGetNumGeoms(dSpaceID space) { return space->count; }
dGeomID dSpaceGetGeom(dSpaceID space, int i) {   // dxSpace::getGeom (collision_space.cpp:131-149)
  // ODE 0.12 leaves the quadtree's enumeration unimplemented (:412-483)
  if (i < 0 || space->qt) return nullptr;
  if (space->sap) {   // dxSAPSpace::getGeom (:293-301): the dirty list, then the clean one
    const int nd = (int)space->sap->dirty.size();
    if (i < nd) return space->sap->dirty[i];
    return i - nd < (int)space->sap->geoms.size() ? space->sap->geoms[i - nd] : nullptr;
  }
  dxGeom* g = space->first;
  for (int j = 0; j < i && g; ++j) g = g->next;
  return g;
}
int dSpaceGetClass(dSpaceID space) { return space->type; }
void dSpaceCollide(dSpaceID space, void* data, dNearCallback* callback) {   // collision_space.cpp:748-753
  if (!space || !callback) return;
  space_collide(space, data, callback);
}
namespace {
struct SwapData { void* data; dNearCallback* cb; };
void swap_callback(void* data, dGeomID g1, dGeomID g2) {   // collision_space.cpp:760-764
  auto* d = static_cast<SwapData*>(data);
  d->cb(d->data, g2, g1);
}
}  // namespace
// dxQuadTreeSpace::collide2 (collision_quadtreespace.cpp:585-611): a member
// against its block and the blocks below, with the pair swapped, then the
// blocks above; any other geom against the whole tree, swapped
static void quad_collide2(dxSpace* sp, void* data, dxGeom* g2, dNearCallback* cb) {
  space_clean(sp);
  recompute_aabb(g2);
  const QuadTree& q = *sp->qt;
  SwapData d{data, cb};
  if (g2->space == sp) {
    int b = g2->qblock;
    quad_collide_geom(q, b, g2, q.blocks[b].first, &d, swap_callback);
    while ((b = q.blocks[b].parent) >= 0)
      for (dxGeom* g1 = q.blocks[b].first; g1; g1 = g1->next)
        if (geom_enabled(g1)) collide_aabbs(g1, g2, data, cb);
  } else {
    quad_collide_geom(q, 0, g2, q.blocks[0].first, &d, swap_callback);
  }
}
// dSpaceCollide2 (collision_space.cpp:767-834): a space against a geom, two
// spaces by the smaller one's members (the deeper sublevel is taken as a
// geom), or two geoms by their boxes alone
void dSpaceCollide2(dGeomID g1, dGeomID g2, void* data, dNearCallback* callback) {
  if (!g1 || !g2 || !callback) return;
  dxSpace* s1 = is_space(g1) ? static_cast<dxSpace*>(g1) : nullptr;
  dxSpace* s2 = is_space(g2) ? static_cast<dxSpace*>(g2) : nullptr;
  if (s1 && s2 && s1->sublevel != s2->sublevel) {
    if (s1->sublevel > s2->sublevel) s2 = nullptr;
    else s1 = nullptr;
  }
  if (s1 && s2) {
    if (s1 == s2) {
      space_collide(s1, data, callback);
    } else if (s1->count < s2->count) {
      SwapData d{data, callback};
      for (dxGeom* g = s1->first; g; g = g->next) space_collide2(s2, &d, g, swap_callback);
    } else {
      for (dxGeom* g = s2->first; g; g = g->next) space_collide2(s1, data, g, callback);
    }
  } else if (s1) {
    space_collide2(s1, data, g2, callback);
  } else if (s2) {
    SwapData d{data, callback};
    space_collide2(s2, &d, g1, swap_callback);
  } else {
    recompute_aabb(g1);
    recompute_aabb(g2);
    collide_aabbs(g1, g2, data, callback);
  }
}

int dCollide(dGeomID o1, dGeomID o2, int flags, dContactGeom* contact, int skip) {
  // early-outs of ode/src/collision_kernel.cpp:292-311, then the collider on the GPU
  if (!o1 || !o2 || !contact || (flags & 0xffff) == 0) return 0;
  if (o1 == o2) return 0;
  if (o1->body == o2->body && o1->body) return 0;
  colliders_init();
  if (o1->type >= 0 && o1->type < kGeomClasses && o2->type >= 0 && o2->type < kGeomClasses &&
      g_colliders[o1->type][o2->type].kind != kColliderBuiltin) {
    // a caller's collider or a user class (collision_kernel.cpp:313-336); a
    // reversed entry swaps the geoms and then flips normals, geoms and sides
    // back
    const ColliderEntry e = g_colliders[o1->type][o2->type];
    dxGeom* a = e.reverse ? o2 : o1;
    dxGeom* b = e.reverse ? o1 : o2;
    int n;
    if (e.kind == kColliderUser) {
      // dCollideUserGeomWithGeom (:940-972): the user geom's class names the
      // collider for the other class, or else the other user class for it;
      // the answer is kept in the table and the pair goes round again
      const int t1 = a->type, t2 = b->type;
      dColliderFn* fn = g_user_classes[t1 - kFirstUserClass].collider(t2);
      int rev = 0;
      if (!fn && is_user_class(t2)) {
        fn = g_user_classes[t2 - kFirstUserClass].collider(t1);
        rev = 1;
      }
      g_colliders[t1][t2] = {kColliderFn, fn, rev};
      g_colliders[t2][t1] = {kColliderFn, fn, !rev};
      n = dCollide(a, b, flags, contact, skip);
    } else if (e.kind == kColliderTransform) {
      // dCollideTransform (collision_transform.cpp:105-150): the wrapped geom
      // collides at the carried pose (the one of the last box, while the
      // transform's box is valid) and with the transform's body; in info
      // mode the contacts name the transform
      dxGeom* o = a->tobj;
      if (!o) return 0;
      if (a->aabb_bad) transform_final(a);
      dxBody* body_bak = o->body;
      o->ovr_pos = a->tpos;
      o->ovr_R = a->tR;
      o->body = a->body;
      n = dCollide(o, b, flags, contact, skip);
      if (a->tinfo)
        for (int i = 0; i < n; ++i) ((dContactGeom*)((char*)contact + (size_t)i * skip))->g1 = a;
      o->ovr_pos = o->ovr_R = nullptr;
      o->body = body_bak;
    } else {
      if (!e.fn) return 0;
      n = e.fn(a, b, flags, contact, skip);
    }
    if (e.reverse)
      for (int i = 0; i < n; ++i) {
        dContactGeom* c = (dContactGeom*)((char*)contact + (size_t)i * skip);
        for (int k = 0; k < 3; ++k) c->normal[k] = -c->normal[k];
        std::swap(c->g1, c->g2);
        std::swap(c->side1, c->side2);
      }
    return n;
  }
  if (is_space(o1) || is_space(o2)) return 0;   // no collider takes a space
  if (o1->type == dHeightfieldClass || o2->type == dHeightfieldClass) {
    // dCollideHeightfield runs with the field first; the reversed call
    // negates the normals (ode/src/collision_kernel.cpp:319-335)
    const bool rev = o2->type == dHeightfieldClass;
    const dxGeom* hg = rev ? o2 : o1;
    const dxGeom* og2 = rev ? o1 : o2;
    if (og2->type != dSphereClass && og2->type != dBoxClass && og2->type != dCapsuleClass &&
        og2->type != dCylinderClass && og2->type != dRayClass)
      return 0;
    if (!hg->hf || !hg->hf->built) return 0;
    double hpos[3] = {0, 0, 0}, hR[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (hg->placeable) {
      const dReal* P = dGeomGetPosition((dGeomID)hg);
      const dReal* R = dGeomGetRotation((dGeomID)hg);
      for (int k = 0; k < 3; ++k) hpos[k] = P[k];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) hR[r * 3 + c] = R[r * 4 + c];
    }
    const dxHeightfieldData* D = hg->hf;
    const og::DevHeightfield H = og::make_dev_heightfield(D->nx, D->nz, D->width, D->depth, D->scale, D->offset,
                                                          D->thickness, D->wrap, hpos, hR, 0);
    og::GeomView gv;
    gv.type = og2->type;
    for (int k = 0; k < 4; ++k) gv.p[k] = (float)og2->p[k];
    const dReal* pos = dGeomGetPosition((dGeomID)og2);
    const dReal* R = dGeomGetRotation((dGeomID)og2);
    for (int k = 0; k < 3; ++k) gv.pos[k] = pos[k];
    for (int k = 0; k < 12; ++k) gv.R[k] = R[k];
    int maxc = flags & 0xffff;
    unsigned f = (unsigned)flags;
    if (maxc > 8) f = (f & ~0xffffu) | 8u;
    og::Contact out[8];
    const int n = og::collide_hf_gpu(H, D->d_heights, gv, f, out);
    if (n <= 0) return 0;
    const float sgn = rev ? -1.f : 1.f;
    for (int i = 0; i < n; ++i) {
      dContactGeom* c = (dContactGeom*)((char*)contact + (size_t)i * skip);
      for (int k = 0; k < 3; ++k) { c->pos[k] = out[i].pos[k]; c->normal[k] = sgn * out[i].normal[k]; }
      c->pos[3] = c->normal[3] = 0;
      c->depth = out[i].depth;
      c->g1 = o1;
      c->g2 = o2;
      c->side1 = c->side2 = -1;
    }
    return n;
  }
  og::GeomView v[2];
  const dxGeom* g[2] = {o1, o2};
  for (int i = 0; i < 2; ++i) {
    v[i].type = g[i]->type;
    for (int k = 0; k < 4; ++k) v[i].p[k] = (float)g[i]->p[k];
    const dReal* pos = dGeomGetPosition((dGeomID)g[i]);
    const dReal* R = dGeomGetRotation((dGeomID)g[i]);
    for (int k = 0; k < 3; ++k) v[i].pos[k] = pos[k];
    for (int k = 0; k < 12; ++k) v[i].R[k] = R[k];
  }
  int maxc = flags & 0xffff;
  unsigned f = (unsigned)flags;
  if (maxc > 8) f = (f & ~0xffffu) | 8u;   // colliders on this path emit at most 8
  og::Contact out[8];
  const int n = og::collide_pair_gpu(v[0], v[1], f, out);
  if (n <= 0) return 0;
  for (int i = 0; i < n; ++i) {
    dContactGeom* c = (dContactGeom*)((char*)contact + (size_t)i * skip);
    for (int k = 0; k < 3; ++k) { c->pos[k] = out[i].pos[k]; c->normal[k] = out[i].normal[k]; }
    c->pos[3] = c->normal[3] = 0;
    c->depth = out[i].depth;
    c->g1 = o1;
    c->g2 = o2;
    c->side1 = c->side2 = -1;
  }
  return n;
}

// ---------------------------------------------------------------- step
static int world_step(dWorldID w, dReal stepsize, bool exact);
int dWorldQuickStep(dWorldID w, dReal stepsize) { return world_step(w, stepsize, false); }
// dWorldStep (ode/src/ode.cpp:1787): the same pipeline with the exact stepper
// of ode/src/step.cpp and its Dantzig LCP on the GPU (world_exact.cuh)
int dWorldStep(dWorldID w, dReal stepsize) { return world_step(w, stepsize, true); }

// dInternalHandleAutoDisabling (ode/src/util.cpp:98-230), the first thing a
// step does: each enabled, auto-disabling body with a joint (no freezing in
// mid-air) samples its velocities into its ring; once the ring is full, an
// average below both thresholds counts the body idle, and idle for the steps
// and the time asked disables it and zeroes its velocities.
static void handle_auto_disabling(dxWorld* w, dReal stepsize) {
  bool any = false;
  for (const dxBody* b : w->bodies) any |= b->auto_disable && !b->disabled;
  if (!any) return;
  std::unordered_map<const dxBody*, char> jointed;
  for (const dxJoint* j : w->joints)
    for (int s = 0; s < 2; ++s)
      if (j->body[s]) jointed[j->body[s]] = 1;
  for (dxBody* b : w->bodies) {
    if (!jointed.count(b) || !b->auto_disable || b->disabled || b->adis_samples == 0) continue;
    if (b->avg_counter >= b->adis_samples) { b->avg_ready = 0; b->avg_counter = 0; }
    dReal* smp = b->avg_buf[b->avg_counter];
    for (int k = 0; k < 3; ++k) { smp[k] = b->lvel[k]; smp[3 + k] = b->avel[k]; }
    if (++b->avg_counter >= b->adis_samples) { b->avg_counter = 0; b->avg_ready = 1; }
    int idle = 0;
    if (b->avg_ready) {
      idle = 1;
      dReal al[3], aa[3];
      for (int k = 0; k < 3; ++k) { al[k] = b->avg_buf[0][k]; aa[k] = b->avg_buf[0][3 + k]; }
      if (b->adis_samples > 1) {
        for (unsigned i = 1; i < b->adis_samples; ++i)
          for (int k = 0; k < 3; ++k) { al[k] += b->avg_buf[i][k]; aa[k] += b->avg_buf[i][3 + k]; }
        const dReal r1 = (dReal)1.0 / (dReal)b->adis_samples;
        for (int k = 0; k < 3; ++k) { al[k] *= r1; aa[k] *= r1; }
      }
      if (al[0] * al[0] + al[1] * al[1] + al[2] * al[2] > b->adis_lin_thr) idle = 0;
      else if (aa[0] * aa[0] + aa[1] * aa[1] + aa[2] * aa[2] > b->adis_ang_thr) idle = 0;
    }
    if (idle) {
      b->adis_stepsleft--;
      b->adis_timeleft -= stepsize;
    } else {
      b->adis_stepsleft = b->adis_steps;
      b->adis_timeleft = b->adis_time;
    }
    if (b->adis_stepsleft <= 0 && b->adis_timeleft <= 0) {
      b->disabled = 1;
      for (int k = 0; k < 3; ++k) b->lvel[k] = b->avel[k] = 0;
    }
  }
}

static int world_step(dWorldID w, dReal stepsize, bool exact) {
  if (!w || !(stepsize > 0)) return 0;
  handle_auto_disabling(w, stepsize);
  if (!w->ctx) {
    w->ctx = og::ctx_create(0);
    if (!w->ctx) return 0;
  }
  og::HostWorld& hw = w->hw;
  // The bodies this step moves (util.cpp:413-470): every enabled body and
  // whatever an enabled joint connects to one, which the island walk enables
  // again; a disabled body reached by none stays as it is, forces included.
  std::vector<dxBody*> sb, woken;
  {
    std::unordered_map<const dxBody*, std::vector<dxBody*>> nbr;
    for (const dxJoint* j : w->joints)
      if (j->body[0] && j->body[1] && !j->disabled) {
        nbr[j->body[0]].push_back(j->body[1]);
        nbr[j->body[1]].push_back(j->body[0]);
      }
    std::unordered_map<const dxBody*, char> reached;
    std::vector<dxBody*> stack;
    for (dxBody* b : w->bodies)
      if (!b->disabled && !reached[b]) {
        reached[b] = 1;
        stack.push_back(b);
        while (!stack.empty()) {
          dxBody* c = stack.back();
          stack.pop_back();
          if (c->disabled) woken.push_back(c);
          c->disabled = 0;
          const auto it = nbr.find(c);
          if (it == nbr.end()) continue;
          for (dxBody* o : it->second)
            if (!reached[o]) { reached[o] = 1; stack.push_back(o); }
        }
      }
    for (dxBody* b : w->bodies)
      if (!b->disabled) sb.push_back(b);
  }
  const int nb = (int)sb.size();
  if (nb == 0) return 1;
  if (nb > ODEGPU_MAX_BODIES_LARGE) return 0;
  hw.pos.resize(nb); hw.q.resize(nb); hw.lvel.resize(nb); hw.avel.resize(nb);
  hw.facc.resize(nb); hw.tacc.resize(nb);
  hw.mass.resize(nb); hw.invMass.resize(nb); hw.I.resize(9 * (size_t)nb); hw.invI.resize(9 * (size_t)nb);
  hw.flags.resize(nb);
  for (int i = 0; i < nb; ++i) {
    dxBody* b = sb[i];
    hw.pos[i] = make_float4(b->pos[0], b->pos[1], b->pos[2], 0.f);
    hw.q[i] = make_float4(b->q[0], b->q[1], b->q[2], b->q[3]);
    hw.lvel[i] = make_float4(b->lvel[0], b->lvel[1], b->lvel[2], 0.f);
    hw.avel[i] = make_float4(b->avel[0], b->avel[1], b->avel[2], 0.f);
    hw.facc[i] = make_float4(b->facc[0], b->facc[1], b->facc[2], 0.f);
    hw.tacc[i] = make_float4(b->tacc[0], b->tacc[1], b->tacc[2], 0.f);
    hw.mass[i] = b->mass.mass;
    hw.invMass[i] = (float)b->invMass;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        hw.I[9 * (size_t)i + r * 3 + c] = b->mass.I[r * 4 + c];
        hw.invI[9 * (size_t)i + r * 3 + c] = (float)b->invI[r * 3 + c];
      }
    hw.flags[i] = b->flags;
  }
  if (!woken.empty()) {   // woken this step: never an island start
    std::unordered_map<const dxBody*, int> slot;
    for (int i = 0; i < nb; ++i) slot[sb[i]] = i;
    for (const dxBody* b : woken) hw.flags[slot[b]] |= og::BODY_WOKEN;
  }
  // dxStepBody options, uploaded only when some body uses one. The finite
  // axis flag without the mode has no effect (util.cpp:272-276).
  bool any_step = false;
  for (const dxBody* b : sb) any_step |= b->step_flags != 0;
  hw.bstep.clear();
  if (any_step) {
    hw.bstep.resize((size_t)og::kStepRec * nb);
    for (int i = 0; i < nb; ++i) {
      const dxBody* b = sb[i];
      float4* r = &hw.bstep[(size_t)og::kStepRec * i];
      int fl = b->step_flags;
      if (!(fl & og::kStepFiniteRot)) fl &= ~og::kStepFiniteAxis;
      float flf;
      std::memcpy(&flf, &fl, sizeof(fl));
      r[0] = make_float4(flf, b->max_angular_speed, b->lin_scale, b->lin_thr);
      r[1] = make_float4(b->ang_scale, b->ang_thr, b->frot_axis[0], b->frot_axis[1]);
      r[2] = make_float4(b->frot_axis[2], 0.f, 0.f, 0.f);
    }
  }
  std::unordered_map<const dxBody*, int> body_index;
  body_index.reserve((size_t)nb);
  for (int i = 0; i < nb; ++i) body_index[sb[i]] = i;
  auto index_of = [&](const dxBody* b) -> int {
    if (!b) return -1;
    const auto it = body_index.find(b);
    return it == body_index.end() ? nb : it->second;
  };
  // joints: persistent first (creation order), then contacts (creation order)
  std::vector<dxJoint*> pj, cj;
  for (dxJoint* j : w->joints) {
    // unattached and disabled joints take no part (util.cpp:435-467, 500-510):
    // they neither join islands nor add rows
    if (!j->body[0] || j->disabled || j->body[0]->disabled) continue;
    (j->type == dJointTypeContact ? cj : pj).push_back(j);
  }
  hw.joints.resize(pj.size());
  for (size_t k = 0; k < pj.size(); ++k) {
    const dxJoint* j = pj[k];
    DevJoint& J = hw.joints[k];
    std::memset(&J, 0, sizeof(J));
    J.type = j->type;
    J.b1 = index_of(j->body[0]);
    J.b2 = index_of(j->body[1]);
    J.reverse = j->reverse;
    og::pack_joint_geometry(j->type, j->h, J);
    J.erp = (float)j->erp; J.cfm = (float)j->cfm;
    J.lm1 = j->lm1; J.lm2 = j->lm2; J.lm3 = j->lm3;
    J.susp_erp = (float)j->susp_erp; J.susp_cfm = (float)j->susp_cfm;
  }
  hw.contacts.resize(cj.size());
  hw.surfaces.resize(std::max<size_t>(1, cj.size()));
  for (size_t k = 0; k < cj.size(); ++k) {
    const dxJoint* j = cj[k];
    DevContact& c = hw.contacts[k];
    std::memset(&c, 0, sizeof(c));
    for (int q = 0; q < 3; ++q) { c.pos[q] = j->contact.geom.pos[q]; c.normal[q] = j->contact.geom.normal[q]; }
    c.depth = j->contact.geom.depth;
    c.surface = (int)k;
    c.b1 = index_of(j->body[0]);
    c.b2 = index_of(j->body[1]);
    c.reverse = j->reverse;
    c.geoms = -1;
    const dSurfaceParameters& S = j->contact.surface;
    DevSurface& D = hw.surfaces[k];
    D.mode = S.mode; D.mu = S.mu; D.mu2 = S.mu2; D.bounce = S.bounce; D.bounce_vel = S.bounce_vel;
    D.soft_erp = S.soft_erp; D.soft_cfm = S.soft_cfm; D.motion1 = S.motion1; D.motion2 = S.motion2;
    D.motionN = S.motionN; D.slip1 = S.slip1; D.slip2 = S.slip2;
  }
  // every body's joint list, newest attachment first
  std::vector<std::vector<std::pair<long long, int>>> lists(nb);
  for (size_t k = 0; k < pj.size(); ++k)
    for (int s = 0; s < 2; ++s)
      if (pj[k]->body[s]) lists[index_of(pj[k]->body[s])].push_back({pj[k]->seq, (int)k});
  for (size_t k = 0; k < cj.size(); ++k)
    for (int s = 0; s < 2; ++s)
      if (cj[k]->body[s]) lists[index_of(cj[k]->body[s])].push_back({cj[k]->seq, (int)(pj.size() + k)});
  hw.padj_start.assign(nb + 1, 0);
  hw.padj.clear();
  for (int i = 0; i < nb; ++i) {
    std::sort(lists[i].begin(), lists[i].end(), [](auto& a, auto& b) { return a.first > b.first; });
    hw.padj_start[i] = (int)hw.padj.size();
    for (auto& e : lists[i]) hw.padj.push_back(e.second);
  }
  hw.padj_start[nb] = (int)hw.padj.size();
  if (hw.padj.empty()) hw.padj.push_back(0);
  og::WorldDesc& D = hw.desc;
  std::memset(&D, 0, sizeof(D));
  D.nb = nb;
  D.njp = (int)pj.size();
  D.contact_cap = (int)cj.size();
  D.row_cap = ODEGPU_MAX_ROWS_PER_WORLD;
  D.iterations = w->iterations;
  for (int k = 0; k < 3; ++k) D.gravity[k] = (float)w->gravity[k];
  D.erp = (float)w->erp; D.cfm = (float)w->cfm; D.sor_w = (float)w->sor_w;
  D.max_vel = (float)w->max_vel; D.min_depth = (float)w->min_depth; D.dt = stepsize;
  D.max_contacts = 1;
  hw.seed = (unsigned)g_seed;
  hw.want_feedback = false;
  for (const dxJoint* j : pj) hw.want_feedback |= j->feedback != nullptr;
  for (const dxJoint* j : cj) hw.want_feedback |= j->feedback != nullptr;
  hw.exact = exact;
  if (og::ctx_step(w->ctx, hw) != 0) return 0;
  g_seed = hw.seed;
  if (hw.want_feedback) {
    // dxQuickStepper fills f1 t1, and f2 t2 when the joint has a second body
    // (ode/src/quickstep.cpp:918-957)
    auto fill = [](dxJoint* j, const float* f) {
      dJointFeedback* fb = j->feedback;
      if (!fb) return;
      for (int q = 0; q < 3; ++q) { fb->f1[q] = f[q]; fb->t1[q] = f[3 + q]; }
      if (j->body[1])
        for (int q = 0; q < 3; ++q) { fb->f2[q] = f[6 + q]; fb->t2[q] = f[9 + q]; }
    };
    for (size_t k = 0; k < pj.size(); ++k) fill(pj[k], hw.feedback.data() + 12 * k);
    for (size_t k = 0; k < cj.size(); ++k) fill(cj[k], hw.contact_feedback.data() + 12 * k);
  }
  for (int i = 0; i < nb; ++i) {
    dxBody* b = sb[i];
    b->pos[0] = hw.pos[i].x; b->pos[1] = hw.pos[i].y; b->pos[2] = hw.pos[i].z;
    b->q[0] = hw.q[i].x; b->q[1] = hw.q[i].y; b->q[2] = hw.q[i].z; b->q[3] = hw.q[i].w;
    body_sync_R(b);
    b->lvel[0] = hw.lvel[i].x; b->lvel[1] = hw.lvel[i].y; b->lvel[2] = hw.lvel[i].z;
    b->avel[0] = hw.avel[i].x; b->avel[1] = hw.avel[i].y; b->avel[2] = hw.avel[i].z;
    for (int k = 0; k < 4; ++k) b->facc[k] = b->tacc[k] = 0;
  }
  // Every stepped body notifies its geoms and then its moved callback
  // (dxStepBody, util.cpp:334-340), body by body in island order
  // (quickstep.cpp:1004-1008, step.cpp:810-812), which moves the geoms to the
  // front of their spaces in that order. The islands
  // are ODE's DFS (util.cpp:413-470): bodies newest first, each body's joints
  // in list order, the bodies found pushed on a stack.
  bool in_order = false;   // geoms in a space, or a moved callback: the order is visible
  for (dxBody* b : sb) {
    in_order |= b->moved_callback != nullptr;
    for (dxGeom* g = b->geom; g && !in_order; g = g->body_next) in_order = g->space != nullptr;
  }
  auto moved = [&](int i) {
    dxBody* b = sb[i];
    body_geoms_moved(b);
    if (b->moved_callback) b->moved_callback(b);
  };
  if (!in_order) {
    for (dxBody* b : sb) body_geoms_moved(b);
  } else {
    const int nj = (int)(pj.size() + cj.size());
    std::vector<int> jb(2 * (size_t)nj);
    for (int k = 0; k < nj; ++k) {
      const dxJoint* j = k < (int)pj.size() ? pj[k] : cj[k - pj.size()];
      jb[2 * k] = index_of(j->body[0]);
      jb[2 * k + 1] = index_of(j->body[1]);
    }
    std::vector<char> btag(nb, 0), jtag(nj, 0);
    std::vector<int> stack;
    for (int first = nb - 1; first >= 0; --first) {
      if (btag[first] || (hw.flags[first] & og::BODY_WOKEN)) continue;
      btag[first] = 1;
      int b = first;
      for (;;) {
        moved(b);
        for (int e = hw.padj_start[b]; e < hw.padj_start[b + 1]; ++e) {
          const int k = hw.padj[e];
          if (jtag[k]) continue;
          jtag[k] = 1;
          const int o = jb[2 * k] == b ? jb[2 * k + 1] : jb[2 * k];
          if (o >= 0 && !btag[o]) {
            btag[o] = 1;
            stack.push_back(o);
          }
        }
        if (stack.empty()) break;
        b = stack.back();
        stack.pop_back();
      }
    }
  }
  return hw.status == 0 ? 1 : 0;
}

}  // extern "C"

// ---------------------------------------------------------------- rotation / vector utilities
// ode/src/rotation.cpp and ode/src/odemath.cpp, in dReal (FP32) arithmetic with
// the reference's operation order, so that a program's set-up code gives the
// values the reference's dSINGLE build gives.
extern "C" {

int dSafeNormalize3(dVector3 a) {   // odemath.cpp:74-117
  const float aa[3] = {std::fabs(a[0]), std::fabs(a[1]), std::fabs(a[2])};
  int idx;
  if (aa[1] > aa[0]) {
    idx = (aa[2] > aa[1]) ? 2 : 1;
  } else if (aa[2] > aa[0]) {
    idx = 2;
  } else {
    if (aa[0] <= 0.f) { a[0] = 1; a[1] = 0; a[2] = 0; return 0; }
    idx = 0;
  }
  a[0] /= aa[idx]; a[1] /= aa[idx]; a[2] /= aa[idx];
  const float l = 1.0f / std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  a[0] *= l; a[1] *= l; a[2] *= l;
  return 1;
}
void dNormalize3(dVector3 a) { dSafeNormalize3(a); }
int dSafeNormalize4(dVector4 a) {   // odemath.cpp:119-138
  float l = a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + a[3] * a[3];
  if (l > 0.f) {
    l = 1.0f / std::sqrt(l);
    a[0] *= l; a[1] *= l; a[2] *= l; a[3] *= l;
    return 1;
  }
  a[0] = 1; a[1] = 0; a[2] = 0; a[3] = 0;
  return 0;
}
void dNormalize4(dVector4 a) { dSafeNormalize4(a); }
void dPlaneSpace(const dVector3 n, dVector3 p, dVector3 q) {   // odemath.cpp:151-178
  if (std::fabs(n[2]) > 0.70710678118654752440f) {
    const float a = n[1] * n[1] + n[2] * n[2];
    const float k = 1.0f / std::sqrt(a);
    p[0] = 0; p[1] = -n[2] * k; p[2] = n[1] * k;
    q[0] = a * k; q[1] = -n[0] * p[2]; q[2] = n[0] * p[1];
  } else {
    const float a = n[0] * n[0] + n[1] * n[1];
    const float k = 1.0f / std::sqrt(a);
    p[0] = -n[1] * k; p[1] = n[0] * k; p[2] = 0;
    q[0] = -n[2] * p[1]; q[1] = n[2] * p[0]; q[2] = a * k;
  }
}
void dRSetIdentity(dMatrix3 R) {
  for (int k = 0; k < 12; ++k) R[k] = 0;
  R[0] = R[5] = R[10] = 1;
}
void dQSetIdentity(dQuaternion q) { q[0] = 1; q[1] = q[2] = q[3] = 0; }
void dQFromAxisAndAngle(dQuaternion q, dReal ax, dReal ay, dReal az, dReal angle) {   // rotation.cpp:169-189
  float l = ax * ax + ay * ay + az * az;
  if (l > 0.f) {
    angle *= 0.5f;
    q[0] = std::cos(angle);
    l = std::sin(angle) * (1.0f / std::sqrt(l));
    q[1] = ax * l; q[2] = ay * l; q[3] = az * l;
  } else {
    dQSetIdentity(q);
  }
}
void dRfromQ(dMatrix3 R, const dQuaternion q) {   // rotation.cpp:236-255
  const float qq1 = 2 * q[1] * q[1], qq2 = 2 * q[2] * q[2], qq3 = 2 * q[3] * q[3];
  R[0] = 1 - qq2 - qq3; R[1] = 2 * (q[1] * q[2] - q[0] * q[3]); R[2] = 2 * (q[1] * q[3] + q[0] * q[2]); R[3] = 0;
  R[4] = 2 * (q[1] * q[2] + q[0] * q[3]); R[5] = 1 - qq1 - qq3; R[6] = 2 * (q[2] * q[3] - q[0] * q[1]); R[7] = 0;
  R[8] = 2 * (q[1] * q[3] - q[0] * q[2]); R[9] = 2 * (q[2] * q[3] + q[0] * q[1]); R[10] = 1 - qq1 - qq2; R[11] = 0;
}
void dRFromAxisAndAngle(dMatrix3 R, dReal ax, dReal ay, dReal az, dReal angle) {
  dQuaternion q;
  dQFromAxisAndAngle(q, ax, ay, az, angle);
  dRfromQ(R, q);
}
void dRFromEulerAngles(dMatrix3 R, dReal phi, dReal theta, dReal psi) {   // rotation.cpp:69-91
  const float sphi = std::sin(phi), cphi = std::cos(phi), stheta = std::sin(theta), ctheta = std::cos(theta);
  const float spsi = std::sin(psi), cpsi = std::cos(psi);
  R[0] = cpsi * ctheta; R[1] = spsi * ctheta; R[2] = -stheta; R[3] = 0;
  R[4] = cpsi * stheta * sphi - spsi * cphi; R[5] = spsi * stheta * sphi + cpsi * cphi; R[6] = ctheta * sphi;
  R[7] = 0;
  R[8] = cpsi * stheta * cphi + spsi * sphi; R[9] = spsi * stheta * cphi - cpsi * sphi; R[10] = ctheta * cphi;
  R[11] = 0;
}
void dRFrom2Axes(dMatrix3 R, dReal ax, dReal ay, dReal az, dReal bx, dReal by, dReal bz) {   // rotation.cpp:94-133
  float l = std::sqrt(ax * ax + ay * ay + az * az);
  if (l <= 0.f) return;
  l = 1.0f / l;
  ax *= l; ay *= l; az *= l;
  const float k = ax * bx + ay * by + az * bz;
  bx -= k * ax; by -= k * ay; bz -= k * az;
  l = std::sqrt(bx * bx + by * by + bz * bz);
  if (l <= 0.f) return;
  l = 1.0f / l;
  bx *= l; by *= l; bz *= l;
  R[0] = ax; R[4] = ay; R[8] = az;
  R[1] = bx; R[5] = by; R[9] = bz;
  R[2] = -by * az + ay * bz; R[6] = -bz * ax + az * bx; R[10] = -bx * ay + ax * by;
  R[3] = R[7] = R[11] = 0;
}
void dRFromZAxis(dMatrix3 R, dReal ax, dReal ay, dReal az) {   // rotation.cpp:136-156
  dVector3 n = {ax, ay, az, 0}, p, q;
  dNormalize3(n);
  dPlaneSpace(n, p, q);
  R[0] = p[0]; R[4] = p[1]; R[8] = p[2];
  R[1] = q[0]; R[5] = q[1]; R[9] = q[2];
  R[2] = n[0]; R[6] = n[1]; R[10] = n[2];
  R[3] = R[7] = R[11] = 0;
}
void dQMultiply0(dQuaternion qa, const dQuaternion qb, const dQuaternion qc) {   // rotation.cpp:191-226
  const float a0 = qb[0] * qc[0] - qb[1] * qc[1] - qb[2] * qc[2] - qb[3] * qc[3];
  const float a1 = qb[0] * qc[1] + qb[1] * qc[0] + qb[2] * qc[3] - qb[3] * qc[2];
  const float a2 = qb[0] * qc[2] + qb[2] * qc[0] + qb[3] * qc[1] - qb[1] * qc[3];
  const float a3 = qb[0] * qc[3] + qb[3] * qc[0] + qb[1] * qc[2] - qb[2] * qc[1];
  qa[0] = a0; qa[1] = a1; qa[2] = a2; qa[3] = a3;
}
void dQMultiply1(dQuaternion qa, const dQuaternion qb, const dQuaternion qc) {
  const float a0 = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
  const float a1 = qb[0] * qc[1] - qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
  const float a2 = qb[0] * qc[2] - qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
  const float a3 = qb[0] * qc[3] - qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
  qa[0] = a0; qa[1] = a1; qa[2] = a2; qa[3] = a3;
}
void dQMultiply2(dQuaternion qa, const dQuaternion qb, const dQuaternion qc) {
  const float a0 = qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2] + qb[3] * qc[3];
  const float a1 = -qb[0] * qc[1] + qb[1] * qc[0] - qb[2] * qc[3] + qb[3] * qc[2];
  const float a2 = -qb[0] * qc[2] + qb[2] * qc[0] - qb[3] * qc[1] + qb[1] * qc[3];
  const float a3 = -qb[0] * qc[3] + qb[3] * qc[0] - qb[1] * qc[2] + qb[2] * qc[1];
  qa[0] = a0; qa[1] = a1; qa[2] = a2; qa[3] = a3;
}
void dQMultiply3(dQuaternion qa, const dQuaternion qb, const dQuaternion qc) {
  const float a0 = qb[0] * qc[0] - qb[1] * qc[1] - qb[2] * qc[2] - qb[3] * qc[3];
  const float a1 = -qb[0] * qc[1] - qb[1] * qc[0] + qb[2] * qc[3] - qb[3] * qc[2];
  const float a2 = -qb[0] * qc[2] - qb[2] * qc[0] + qb[3] * qc[1] - qb[1] * qc[3];
  const float a3 = -qb[0] * qc[3] - qb[3] * qc[0] + qb[1] * qc[2] - qb[2] * qc[1];
  qa[0] = a0; qa[1] = a1; qa[2] = a2; qa[3] = a3;
}
void dQfromR(dQuaternion q, const dMatrix3 R) {   // rotation.cpp:258-306
  const float tr = R[0] + R[5] + R[10];
  float s;
  if (tr >= 0) {
    s = std::sqrt(tr + 1);
    q[0] = 0.5f * s;
    s = 0.5f * (1.0f / s);
    q[1] = (R[9] - R[6]) * s; q[2] = (R[2] - R[8]) * s; q[3] = (R[4] - R[1]) * s;
    return;
  }
  const int c = (R[5] > R[0]) ? ((R[10] > R[5]) ? 2 : 1) : ((R[10] > R[0]) ? 2 : 0);
  if (c == 0) {
    s = std::sqrt((R[0] - (R[5] + R[10])) + 1);
    q[1] = 0.5f * s;
    s = 0.5f * (1.0f / s);
    q[2] = (R[1] + R[4]) * s; q[3] = (R[8] + R[2]) * s; q[0] = (R[9] - R[6]) * s;
  } else if (c == 1) {
    s = std::sqrt((R[5] - (R[10] + R[0])) + 1);
    q[2] = 0.5f * s;
    s = 0.5f * (1.0f / s);
    q[3] = (R[6] + R[9]) * s; q[1] = (R[1] + R[4]) * s; q[0] = (R[2] - R[8]) * s;
  } else {
    s = std::sqrt((R[10] - (R[0] + R[5])) + 1);
    q[3] = 0.5f * s;
    s = 0.5f * (1.0f / s);
    q[1] = (R[8] + R[2]) * s; q[2] = (R[6] + R[9]) * s; q[0] = (R[4] - R[1]) * s;
  }
}
void dDQfromW(dReal dq[4], const dVector3 w, const dQuaternion q) {   // rotation.cpp:310-317
  dq[0] = 0.5f * (-w[0] * q[1] - w[1] * q[2] - w[2] * q[3]);
  dq[1] = 0.5f * (w[0] * q[0] + w[1] * q[3] - w[2] * q[2]);
  dq[2] = 0.5f * (-w[0] * q[3] + w[1] * q[0] + w[2] * q[1]);
  dq[3] = 0.5f * (w[0] * q[2] - w[1] * q[1] + w[2] * q[0]);
}

}  // extern "C"

// ---------------------------------------------------------------- user data, body helpers, mass algebra
extern "C" {

void dBodySetData(dBodyID b, void* data) { b->data = data; }               // ode.cpp:305-316
void* dBodyGetData(dBodyID b) { return b->data; }
void dGeomSetData(dGeomID g, void* data) { g->data = data; }               // collision_kernel.cpp:386-399
void* dGeomGetData(dGeomID g) { return g->data; }
void dJointSetData(dJointID j, void* data) { j->data = data; }             // ode.cpp:1262-1273
void* dJointGetData(dJointID j) { return j->data; }

// dAreConnected (ode.cpp:1518-1526): a joint of any type attaches the two;
// b2 = 0 asks for a joint to the static environment
int dAreConnected(dBodyID b1, dBodyID b2) {
  if (!b1) return 0;
  for (const dxJoint* j : b1->world->joints)
    if ((j->body[0] == b1 && j->body[1] == b2) || (j->body[1] == b1 && j->body[0] == b2)) return 1;
  return 0;
}
// dBodyGetNumJoints / dBodyGetJoint (ode.cpp:735-758): the body's joints in its
// list order, newest attachment first
static std::vector<dxJoint*> body_joints(dBodyID b) {
  std::vector<dxJoint*> js;
  for (dxJoint* j : b->world->joints)
    if (j->body[0] == b || j->body[1] == b) js.push_back(j);
  std::stable_sort(js.begin(), js.end(), [](const dxJoint* x, const dxJoint* y) { return x->seq > y->seq; });
  return js;
}
int dBodyGetNumJoints(dBodyID b) { return b ? (int)body_joints(b).size() : 0; }
dJointID dBodyGetJoint(dBodyID b, int index) {
  if (!b || index < 0) return nullptr;
  const auto js = body_joints(b);
  return index < (int)js.size() ? js[index] : nullptr;
}

// body-frame vectors and points in world coordinates (ode.cpp:645-733)
static void body_rot(const dxBody* b, const float* v, float* out) {
  for (int i = 0; i < 3; ++i) out[i] = b->R[i * 4 + 0] * v[0] + b->R[i * 4 + 1] * v[1] + b->R[i * 4 + 2] * v[2];
}
void dBodyVectorToWorld(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result) {
  const float p[3] = {px, py, pz};
  body_rot(b, p, result);
}
void dBodyGetRelPointPos(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result) {
  const float p[3] = {px, py, pz};
  body_rot(b, p, result);
  for (int i = 0; i < 3; ++i) result[i] += b->pos[i];
}
void dBodyVectorFromWorld(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result) {   // ode.cpp:757-770
  for (int i = 0; i < 3; ++i) result[i] = b->R[0 * 4 + i] * px + b->R[1 * 4 + i] * py + b->R[2 * 4 + i] * pz;
}
void dBodyGetPosRelPoint(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result) {    // ode.cpp:728-741
  dBodyVectorFromWorld(b, px - b->pos[0], py - b->pos[1], pz - b->pos[2], result);
}
// velocity of a body point: v + w x (p - pos) (ode.cpp:696-726)
void dBodyGetRelPointVel(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result) {
  float q[3];
  const float p[3] = {px, py, pz};
  body_rot(b, p, q);
  const float* w = b->avel;
  result[0] = b->lvel[0] + w[1] * q[2] - w[2] * q[1];
  result[1] = b->lvel[1] + w[2] * q[0] - w[0] * q[2];
  result[2] = b->lvel[2] + w[0] * q[1] - w[1] * q[0];
}
void dBodyGetPointVel(dBodyID b, dReal px, dReal py, dReal pz, dVector3 result) {
  const float q[3] = {px - b->pos[0], py - b->pos[1], pz - b->pos[2]};
  const float* w = b->avel;
  result[0] = b->lvel[0] + w[1] * q[2] - w[2] * q[1];
  result[1] = b->lvel[1] + w[2] * q[0] - w[0] * q[2];
  result[2] = b->lvel[2] + w[0] * q[1] - w[1] * q[0];
}
void dBodySetForce(dBodyID b, dReal x, dReal y, dReal z) { b->facc[0] = x; b->facc[1] = y; b->facc[2] = z; }   // ode.cpp:656-663
void dBodySetTorque(dBodyID b, dReal x, dReal y, dReal z) { b->tacc[0] = x; b->tacc[1] = y; b->tacc[2] = z; }

// force helpers (ode.cpp:537-641): forces and torques in world coordinates
// into the accumulators
void dBodyAddRelForce(dBodyID b, dReal fx, dReal fy, dReal fz) {
  const float f[3] = {fx, fy, fz};
  float w[3];
  body_rot(b, f, w);
  for (int i = 0; i < 3; ++i) b->facc[i] += w[i];
}
void dBodyAddRelTorque(dBodyID b, dReal fx, dReal fy, dReal fz) {
  const float f[3] = {fx, fy, fz};
  float w[3];
  body_rot(b, f, w);
  for (int i = 0; i < 3; ++i) b->tacc[i] += w[i];
}
static void add_force_at(dxBody* b, const float* f, const float* p) {
  const float q[3] = {p[0] - b->pos[0], p[1] - b->pos[1], p[2] - b->pos[2]};
  for (int i = 0; i < 3; ++i) b->facc[i] += f[i];
  b->tacc[0] += q[1] * f[2] - q[2] * f[1];
  b->tacc[1] += q[2] * f[0] - q[0] * f[2];
  b->tacc[2] += q[0] * f[1] - q[1] * f[0];
}
void dBodyAddForceAtPos(dBodyID b, dReal fx, dReal fy, dReal fz, dReal px, dReal py, dReal pz) {
  const float f[3] = {fx, fy, fz}, p[3] = {px, py, pz};
  add_force_at(b, f, p);
}
void dBodyAddForceAtRelPos(dBodyID b, dReal fx, dReal fy, dReal fz, dReal px, dReal py, dReal pz) {
  const float f[3] = {fx, fy, fz};
  float p[3];
  dBodyGetRelPointPos(b, px, py, pz, p);
  add_force_at(b, f, p);
}
void dBodyAddRelForceAtPos(dBodyID b, dReal fx, dReal fy, dReal fz, dReal px, dReal py, dReal pz) {
  const float fl[3] = {fx, fy, fz}, p[3] = {px, py, pz};
  float f[3];
  body_rot(b, fl, f);
  add_force_at(b, f, p);
}
void dBodyAddRelForceAtRelPos(dBodyID b, dReal fx, dReal fy, dReal fz, dReal px, dReal py, dReal pz) {
  const float fl[3] = {fx, fy, fz};
  float f[3], p[3];
  body_rot(b, fl, f);
  dBodyGetRelPointPos(b, px, py, pz, p);
  add_force_at(b, f, p);
}

// mass algebra (ode/src/mass.cpp:454-537)
static void mul0_333f(float* A, const float* B, const float* C) {   // A = B C (3x4 rows)
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j)
      A[i * 4 + j] = B[i * 4 + 0] * C[0 * 4 + j] + B[i * 4 + 1] * C[1 * 4 + j] + B[i * 4 + 2] * C[2 * 4 + j];
    A[i * 4 + 3] = 0;
  }
}
static void cross_mat(float* A, const float* a) {   // A v = a x v
  for (int k = 0; k < 12; ++k) A[k] = 0;
  A[1] = -a[2]; A[2] = a[1];
  A[4] = a[2]; A[6] = -a[0];
  A[8] = -a[1]; A[9] = a[0];
}
void dMassTranslate(dMass* m, dReal x, dReal y, dReal z) {
  // I + mass (crossmat(c)^2 - crossmat(c + a)^2), then c += a
  float chat[12], ahat[12], t1[12], t2[12];
  cross_mat(chat, m->c);
  const float a[3] = {x + m->c[0], y + m->c[1], z + m->c[2]};
  cross_mat(ahat, a);
  mul0_333f(t1, ahat, ahat);
  mul0_333f(t2, chat, chat);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) m->I[i * 4 + j] += m->mass * (t2[i * 4 + j] - t1[i * 4 + j]);
  m->I[4] = m->I[1]; m->I[8] = m->I[2]; m->I[9] = m->I[6];
  m->c[0] += x; m->c[1] += y; m->c[2] += z;
}
void dMassRotate(dMass* m, const dMatrix3 R) {
  // R I R', c = R c
  float t1[12], RT[12];
  for (int i = 0; i < 3; ++i) { for (int j = 0; j < 3; ++j) RT[i * 4 + j] = R[j * 4 + i]; RT[i * 4 + 3] = 0; }
  mul0_333f(t1, m->I, RT);
  mul0_333f(m->I, R, t1);
  m->I[4] = m->I[1]; m->I[8] = m->I[2]; m->I[9] = m->I[6];
  float t2[3];
  for (int i = 0; i < 3; ++i) t2[i] = R[i * 4 + 0] * m->c[0] + R[i * 4 + 1] * m->c[1] + R[i * 4 + 2] * m->c[2];
  m->c[0] = t2[0]; m->c[1] = t2[1]; m->c[2] = t2[2];
}
// Cholesky test of a 3x3 (row stride 4) over its lower triangle, as
// dIsPositiveDefinite does (matrix.cpp:124-160, 226-238): positive definite
// when every pivot's reduced diagonal stays above 0
static int positive_definite3(const float* A) {
  float L[12], recip[3];
  for (int k = 0; k < 12; ++k) L[k] = A[k];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < i; ++j) {
      float sum = L[i * 4 + j];
      for (int k = 0; k < j; ++k) sum -= L[i * 4 + k] * L[j * 4 + k];
      L[i * 4 + j] = sum * recip[j];
    }
    float sum = L[i * 4 + i];
    for (int k = 0; k < i; ++k) sum -= L[i * 4 + k] * L[i * 4 + k];
    if (sum <= 0.0f) return 0;
    L[i * 4 + i] = std::sqrt(sum);
    recip[i] = 1.0f / L[i * 4 + i];
  }
  return 1;
}
// dMassCheck (mass.cpp:44-83): mass > 0, I positive definite, and the
// inertia about the centre of mass, I + mass crossmat(c)^2, as well. The
// mass test is the reference's `mass <= 0`, so a NaN mass goes on to the
// inertia tests as it does there.
int dMassCheck(const dMass* m) {
  if (m->mass <= 0) return 0;
  if (!positive_definite3(m->I)) return 0;
  float chat[12], I2[12];
  cross_mat(chat, m->c);
  mul0_333f(I2, chat, chat);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) I2[i * 4 + j] = m->I[i * 4 + j] + m->mass * I2[i * 4 + j];
  return positive_definite3(I2);
}
void dMassAdd(dMass* a, const dMass* b) {
  const float denom = 1.0f / (a->mass + b->mass);
  for (int i = 0; i < 3; ++i) a->c[i] = (a->c[i] * a->mass + b->c[i] * b->mass) * denom;
  a->mass += b->mass;
  for (int i = 0; i < 12; ++i) a->I[i] += b->I[i];
}

}  // extern "C"

// ---------------------------------------------------------------- small accessors
extern "C" {

void dBodyCopyPosition(dBodyID b, dVector3 pos) { for (int k = 0; k < 3; ++k) pos[k] = b->pos[k]; }   // ode.cpp:410-440
void dBodyCopyRotation(dBodyID b, dMatrix3 R) { for (int k = 0; k < 12; ++k) R[k] = b->R[k]; }
void dBodyCopyQuaternion(dBodyID b, dQuaternion q) { for (int k = 0; k < 4; ++k) q[k] = b->q[k]; }
dWorldID dBodyGetWorld(dBodyID b) { return b->world; }                                         // ode.cpp:333-337
// ode.cpp:1399-1410: 0 for a detached joint, 1 for a joint to the environment
int dJointGetNumBodies(dJointID j) { return !j->body[0] ? 0 : (!j->body[1] ? 1 : 2); }
// dConnectingJoint / dConnectingJointList (ode.cpp:1466-1515): the joints
// joining b1 to b2 (0 = the environment) in b1's list order, newest first
dJointID dConnectingJoint(dBodyID in_b1, dBodyID in_b2) {
  dBodyID b1 = in_b1 ? in_b1 : in_b2, b2 = in_b1 ? in_b2 : in_b1;
  if (!b1) return nullptr;
  for (dxJoint* j : body_joints(b1))
    if ((j->body[0] == b1 && j->body[1] == b2) || (j->body[1] == b1 && j->body[0] == b2)) return j;
  return nullptr;
}
int dConnectingJointList(dBodyID in_b1, dBodyID in_b2, dJointID* out) {
  dBodyID b1 = in_b1 ? in_b1 : in_b2, b2 = in_b1 ? in_b2 : in_b1;
  if (!b1) return 0;
  int n = 0;
  for (dxJoint* j : body_joints(b1))
    if ((j->body[0] == b1 && j->body[1] == b2) || (j->body[1] == b1 && j->body[0] == b2)) out[n++] = j;
  return n;
}
// ode.cpp:1783-1791
void dWorldImpulseToForce(dWorldID, dReal stepsize, dReal ix, dReal iy, dReal iz, dVector3 force) {
  const float s = 1.0f / stepsize;
  force[0] = s * ix; force[1] = s * iy; force[2] = s * iz;
}
// misc.cpp:57-60
dReal dRandReal(void) { return (dReal)dRand() / (dReal)0xffffffffUL; }

// Matrix helpers of ode/src/misc.cpp:139-195 over row-padded matrices
// (rows of dPAD(columns) entries, include/ode/common.h:136)
static int pad4(int a) { return a > 1 ? ((a - 1) | 3) + 1 : a; }
void dPrintMatrix(const dReal* A, int n, int m, const char* fmt, FILE* f) {   // misc.cpp:128-136
  const int skip = pad4(m);
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < m; ++j) std::fprintf(f, fmt, A[(size_t)i * skip + j]);
    std::fprintf(f, "\n");
  }
}
void dMakeRandomVector(dReal* A, int n, dReal range) {
  for (int i = 0; i < n; ++i) A[i] = (dRandReal() * (dReal)2.0 - (dReal)1.0) * range;
}
void dMakeRandomMatrix(dReal* A, int n, int m, dReal range) {
  const int skip = pad4(m);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j) A[(size_t)i * skip + j] = (dRandReal() * (dReal)2.0 - (dReal)1.0) * range;
}
void dClearUpperTriangle(dReal* A, int n) {
  const int skip = pad4(n);
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) A[(size_t)i * skip + j] = 0;
}
dReal dMaxDifference(const dReal* A, const dReal* B, int n, int m) {
  const int skip = pad4(m);
  dReal mx = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j) {
      const dReal d = std::fabs(A[(size_t)i * skip + j] - B[(size_t)i * skip + j]);
      if (d > mx) mx = d;
    }
  return mx;
}
dReal dMaxDifferenceLowerTriangle(const dReal* A, const dReal* B, int n) {
  const int skip = pad4(n);
  dReal mx = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      const dReal d = std::fabs(A[(size_t)i * skip + j] - B[(size_t)i * skip + j]);
      if (d > mx) mx = d;
    }
  return mx;
}
// dOrthogonalizeR (ode/src/odemath.cpp:187-211): rows 0 and 1 normalised
// (row 1 first made orthogonal to row 0 by a Gram-Schmidt step), row 2 their
// cross product, so the result is a rotation and never a reflection
void dOrthogonalizeR(dMatrix3 m) {
  if (m[0] * m[0] + m[1] * m[1] + m[2] * m[2] != 1) dSafeNormalize3(m);
  const dReal proj = m[0] * m[4] + m[1] * m[5] + m[2] * m[6];
  if (proj != 0) {
    m[4] -= proj * m[0];
    m[5] -= proj * m[1];
    m[6] -= proj * m[2];
  }
  if (m[4] * m[4] + m[5] * m[5] + m[6] * m[6] != 1) dSafeNormalize3(m + 4);
  m[8] = m[1] * m[6] - m[2] * m[5];
  m[9] = m[2] * m[4] - m[0] * m[6];
  m[10] = m[0] * m[5] - m[1] * m[4];
  m[3] = m[7] = m[11] = 0;
}
// the pre-0.9 names of the capsule mass functions (mass.cpp:544-553)
void dMassSetCappedCylinder(dMass* m, dReal density, int direction, dReal radius, dReal length) {
  dMassSetCapsule(m, density, direction, radius, length);
}
void dMassSetCappedCylinderTotal(dMass* m, dReal total_mass, int direction, dReal radius, dReal length) {
  dMassSetCapsuleTotal(m, total_mass, direction, radius, length);
}
void dJointGetBallAnchor2(dJointID j, dVector3 r) { joint_anchor(j, true, r); }          // ball.cpp:103-113
void dJointGetUniversalAnchor2(dJointID j, dVector3 r) { joint_anchor(j, true, r); }     // universal.cpp:572-582
// ball.cpp:128-143: ERP and CFM only
dReal dJointGetBallParam(dJointID j, int p) {
  return p == dParamCFM ? (dReal)j->cfm : (p == dParamERP ? (dReal)j->erp : 0);
}
// ode.cpp:1401-1417
void dJointEnable(dJointID j) { j->disabled = 0; }
void dJointDisable(dJointID j) { j->disabled = 1; }
int dJointIsEnabled(dJointID j) { return !j->disabled; }
dReal dJointGetHingeParam(dJointID j, int p) { return limot_get(j->lm1, p); }             // hinge.cpp:260-266
dReal dJointGetHinge2Param(dJointID j, int p) {                                           // hinge2.cpp:278-299
  if ((p & 0xff00) == 0x100) return limot_get(j->lm2, p & 0xff);
  if (p == dParamSuspensionERP) return (dReal)j->susp_erp;
  if (p == dParamSuspensionCFM) return (dReal)j->susp_cfm;
  return limot_get(j->lm1, p);
}

}  // extern "C"
