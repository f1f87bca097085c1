/*
 * odegpu.h -- C ABI of libodegpu: the batched world-stepping extension.
 *
 * A batch holds many independent ODE worlds resident in GPU memory and steps
 * them with the CUDA path: contact generation by the primitive colliders
 * (dCollide, ode/src/collision_kernel.cpp:292) in the canonical pair order of
 * odegpu_scene.h, then dWorldQuickStep (ode/src/ode.cpp:1807-1824) per world.
 * Plain pointers and sizes only. All functions return 0 on success and a
 * negative ODEGPU_E* code on failure; odegpuGetLastError() describes the last
 * failure on the calling thread. The ODE-compatible single-world API lives in
 * ode_gpu.h.
 */
#ifndef ODEGPU_H
#define ODEGPU_H
#include <stddef.h>
#include "odegpu_scene.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ODEGPU_OK = 0,
  ODEGPU_E_ARG = -1,       /* invalid argument                                */
  ODEGPU_E_CUDA = -2,      /* CUDA runtime error (no device, launch failure)  */
  ODEGPU_E_NOMEM = -3,     /* device allocation failed                        */
  ODEGPU_E_LIMIT = -4      /* a world exceeds a documented size limit         */
};

/* Per-world status bits reported by odegpuBatchGetStatus. */
enum {
  ODEGPU_ST_CONTACT_OVERFLOW = 1,
  ODEGPU_ST_ROW_OVERFLOW = 2,
  ODEGPU_ST_TOO_LARGE = 4,
  ODEGPU_ST_NONFINITE = 8,
  /* a geom covered more heightfield samples than the collider holds (10 x 10
     in the lane, or the world's workspace, at most 128 x 128, for worlds
     whose geoms can cover more than 10 samples per axis); that pair produced
     no contacts in the step */
  ODEGPU_ST_HF_ZONE = 32,
  /* large world: a geom had more than 64 candidate partners, or the
     candidate pairs exceeded the batch's pair capacity; pairs were dropped */
  ODEGPU_ST_PAIR_OVERFLOW = 64,
  /* large world: a wait of the constraint sweep gave up (bounded); the step's
     constraint forces are incomplete */
  ODEGPU_ST_SOLVE_STALL = 128,
  /* dWorldStep: the LCP solver stopped on a non-positive step, as the
   * reference does (ode/src/lcp.cpp:985-993), or after a bounded number of
   * index-set changes for one driving index */
  ODEGPU_ST_LCP_STOP = 256
};

/* Size limits of the on-chip step kernel: bodies and constraint rows per
 * world. A batch with a single world may exceed them: that world is stepped
 * by the large-world pipeline (every kernel spread over the GPU), up to
 * ODEGPU_MAX_BODIES_LARGE bodies. */
#define ODEGPU_MAX_BODIES_PER_WORLD 64
#define ODEGPU_MAX_ROWS_PER_WORLD 1024
#define ODEGPU_MAX_BODIES_LARGE 65536

typedef struct odegpuBatch* odegpuBatchID;

typedef struct odegpuBatchConfig {
  int contacts_per_body;   /* contact capacity per world = this * nb + 16 (0 -> 8) */
  int warps_per_block;     /* 0 -> chosen by the library                          */
  int device;              /* CUDA device ordinal                                 */
  int large_world;         /* 1: step the batch's single world with the large-world
                              pipeline even when it fits the on-chip kernel     */
} odegpuBatchConfig;

/* Diagnostics of a large-world batch, accumulated since creation or the last
 * reset (reset != 0 clears them after reading): out[0] ns in the island walk,
 * out[1] ns in the sweeps' first iterations, out[2] ns sorting rows by
 * dependency level, out[3] ns in the remaining iterations, out[4] the largest
 * level count met, out[5] sweep launches, out[6] island walks, out[7] ns of
 * the walks spent staging their arrays on chip, out[8] the sweep cluster's
 * CTA count. No counterpart in the reference. */
int odegpuBatchLargeWorldStats(odegpuBatchID b, long long* out, int n, int reset);

/* Body state record used by the read/write calls: pos[3] q[4] lvel[3] avel[3]. */
#define ODEGPU_BODY_REC 13

/* Create a batch from a scene (copied; the scene may be freed afterwards).
 * Replaces building each world with dWorldCreate, dBodyCreate, the dCreate
 * geom constructors and the dJointCreate calls (include/ode/objects.h,
 * include/ode/collision.h). */
int odegpuBatchCreate(const odegpuScene* scene, const odegpuBatchConfig* cfg,
                      odegpuBatchID* out);
void odegpuBatchDestroy(odegpuBatchID b);

/* Enqueue n_steps full steps (collide + QuickStep) of every world on the
 * batch's stream, all steps in one launch. Replaces, per world and step, the
 * dSpaceCollide/dCollide + dJointCreateContact + dWorldQuickStep +
 * dJointGroupEmpty sequence (ode/src/ode.cpp:1201, :1807, :1305). */
int odegpuBatchStep(odegpuBatchID b, int n_steps);
/* Same work as odegpuBatchStep but one world per launch (the plain, unbatched
 * GPU path used as a comparator). */
int odegpuBatchStepPlain(odegpuBatchID b, int n_steps);
/* Capture n_steps single-step launches into a CUDA graph and replay it. */
int odegpuBatchStepGraph(odegpuBatchID b, int n_steps);
/* The stepper every step entry point uses from now on: 0 dWorldQuickStep
 * (ode/src/ode.cpp:1807), 1 dWorldStep (ode/src/ode.cpp:1787; ode/src/step.cpp
 * with the Dantzig LCP of ode/src/lcp.cpp). dWorldStep works on dense
 * m x m matrices per island: each step sizes a world's scratch (about
 * 8 m^2 bytes) by the rows its joints and that step's contacts can need
 * (3 per contact, 6 per persistent joint), reads the total back once and
 * grows a shared arena when it is short. A captured graph cannot read back,
 * so odegpuBatchStepGraph under dWorldStep first lays the arena out by
 * every world's row capacity (up to 1024 rows: ~8 MB per world). dWorldStep
 * is not available for a large world, the parity taps, the adjoint or the
 * autotuner. */
int odegpuBatchSetStepper(odegpuBatchID b, int exact);
int odegpuBatchSynchronize(odegpuBatchID b);

/* Per-step controls from FP32 arrays in host or device memory (the layout
 * of odegpuBatchSetControls); null leaves that kind of control off. */
int odegpuBatchSetControlsF32(odegpuBatchID b, int n_ctrl_steps, const float* joint_torque,
                              const float* body_force);

/* Differentiation (no counterpart in the reference: ODE has no gradients).
 * RolloutForward steps every world n_steps times from the current state like
 * odegpuBatchStep, recording the state and RNG seeds every ckpt_every steps.
 * RolloutBackward takes d(loss)/d(final state) ([nb_total][ODEGPU_BODY_REC]
 * FP32, host or device memory) and writes d(loss)/d(initial state) (same
 * layout), d(loss)/d(joint torques) ([n_ctrl_steps][nj_total][2]) and
 * d(loss)/d(body forces) ([n_ctrl_steps][nb_total][6]); any output may be
 * null. It recomputes each checkpoint segment and runs the hand-written
 * adjoint of every step backwards (one warp per world), then leaves the
 * batch in the state the forward rollout ended in. The derivative follows
 * the recorded active set of the sweep (clamped rows pass nothing to their
 * own lambda). AdjointStatus returns per-world bits, each for a part whose
 * derivative is left out: 1 a joint the adjoint does not model (slider,
 * universal, fixed, angular motor, hinge2 without a second body) or a limit
 * row that bounces or has a powered motor pushing against it; 2 a contact it
 * does not model (a bouncing contact, a fixed friction direction, a capsule
 * or cylinder vertex on a heightfield, a geom under a heightfield); 4 the
 * world exceeds the kernel's limits; 8 a contact between two bodies whose
 * collider answer changes case within every difference step (the geometry
 * Jacobian of such contacts is a central difference of the FP32 collider). */
int odegpuBatchRolloutForward(odegpuBatchID b, int n_steps, int ckpt_every);
int odegpuBatchRolloutBackward(odegpuBatchID b, const float* grad_state_final, float* grad_state_init,
                               float* grad_joint_torque, float* grad_body_force);
int odegpuBatchAdjointStatus(odegpuBatchID b, int* status);

/* Launch shape of each kernel (no counterpart in the reference): kernel 0
 * collide, 1 setup, 2 solve, 3 adjoint, 4 the fused step kernel; warps per
 * block (one world per warp; at most 4, 8, 8, 4, 4) and the preferred
 * shared-memory carveout in percent of the unified L1/shared array (-1 =
 * driver default). GetLaunchConfig writes cfg[8] = {wpb, carveout} of
 * kernels 0-3; GetStepKernels reports kernel 4.
 * SetStepKernels(fused): a step is one launch of the fused step kernel
 * (fused = 1: every warp runs collide, setup and solve of its world in turn,
 * so short worlds do not wait at phase boundaries for the long ones) or the
 * collide, setup and solve kernels (fused = 0, the default until Autotune
 * picks). Both give the same results. With timing on (SetTiming), a fused
 * step's time is reported in the collide entry of GetKernelTimes.
 * Autotune times n_steps steps of every candidate shape on the batch's
 * current state (restored after each trial), keeps the fastest per kernel and
 * chooses fused or split steps by the faster step; the batch state, seeds and
 * step index are unchanged afterwards. */
int odegpuBatchSetLaunchConfig(odegpuBatchID b, int kernel, int warps_per_block, int smem_carveout);
int odegpuBatchGetLaunchConfig(odegpuBatchID b, int* cfg);
/* The same with a kernel variant: variant 1 of the solve kernel (2) caps it
 * at 128 registers per thread, for 16 warps per SM instead of 12 (batches of
 * small worlds gain from the occupancy, batches of large ones lose to the
 * spills); every other kernel has variant 0 only. Autotune also picks the
 * solve kernel's variant. */
int odegpuBatchSetLaunchConfigEx(odegpuBatchID b, int kernel, int warps_per_block, int smem_carveout,
                                 int variant);
int odegpuBatchGetLaunchConfigEx(odegpuBatchID b, int kernel, int* warps_per_block, int* smem_carveout,
                                 int* variant);
int odegpuBatchSetStepKernels(odegpuBatchID b, int fused);
int odegpuBatchGetStepKernels(odegpuBatchID b, int* fused, int* warps_per_block, int* smem_carveout);
int odegpuBatchAutotune(odegpuBatchID b, int n_steps);

/* Instrumentation (no counterpart in the reference).
 * SetTiming(on) makes every following non-graph step record CUDA events on
 * the batch stream around its three kernels (collide, setup, solve) and
 * clears earlier records. GetKernelTimes synchronises the stream, returns
 * the summed milliseconds of each kernel since the last call (ms[3]) and the
 * number of steps they cover, and clears the records. GetLaunchCount
 * returns how many kernels the batch has launched since creation. */
int odegpuBatchSetTiming(odegpuBatchID b, int on);
int odegpuBatchGetKernelTimes(odegpuBatchID b, double* ms, long long* n_steps);
int odegpuBatchGetLaunchCount(odegpuBatchID b, long long* launches);

/* Body state exchange with host memory (FP64 records of ODEGPU_BODY_REC).
 * Read = dBodyGetPosition/Quaternion/LinearVel/AngularVel over all bodies;
 * write = dBodySetPosition/Quaternion/LinearVel/AngularVel. */
int odegpuBatchReadState(odegpuBatchID b, double* state);
int odegpuBatchWriteState(odegpuBatchID b, const double* state);
/* FP32 variants for pinned-host or device buffers, enqueued on the stream
 * without synchronising: float state[nb_total][ODEGPU_BODY_REC]. */
int odegpuBatchReadStateF32Async(odegpuBatchID b, float* state);
int odegpuBatchWriteStateF32Async(odegpuBatchID b, const float* state);

/* Joint feedback (dJointSetFeedback, include/ode/objects.h; filled by
 * dxQuickStepper at ode/src/quickstep.cpp:918-957): SetFeedback(1) makes
 * every following step compute, for every persistent joint, f1 t1 f2 t2 =
 * J^T lambda of its rows (f2 = t2 = 0 without a second body); GetFeedback
 * copies the last step's values to out[nj_total][12] (f1[3] t1[3] f2[3] t2[3]).
 * Both steppers and both pipelines (worlds on one warp each, and the
 * large-world pipeline) fill it. */
int odegpuBatchSetFeedback(odegpuBatchID b, int on);
int odegpuBatchGetFeedback(odegpuBatchID b, double* out);

/* Per-world bookkeeping of the last step. */
int odegpuBatchGetStatus(odegpuBatchID b, int* status);
int odegpuBatchGetCounts(odegpuBatchID b, int* ncontacts, int* nrows, int* nislands);
int odegpuBatchGetSeeds(odegpuBatchID b, unsigned int* seeds);
/* dRandSetSeed per world (the reference has one global seed; a batch has one
 * per world). */
int odegpuBatchSetSeeds(odegpuBatchID b, const unsigned int* seeds);
int odegpuBatchInfo(odegpuBatchID b, int* n_worlds, int* nb_total, int* nj_total,
                    long long* row_capacity, long long* contact_capacity);
/* The CUDA stream the batch enqueues on (a cudaStream_t). */
void* odegpuBatchStream(odegpuBatchID b);

/* Replace the per-step controls (same layout as odegpuScene): joint_torque
 * [n_ctrl_steps][nj_total][2], body_force [n_ctrl_steps][nb_total][6]; either
 * may be NULL. Replaces dJointAddHingeTorque / dJointAddHinge2Torques /
 * dBodyAddForce / dBodyAddTorque calls made before each step. */
int odegpuBatchSetControls(odegpuBatchID b, int n_ctrl_steps, const double* joint_torque,
                           const double* body_force);
/* Replace the per-step joint stops (layout of odegpuScene::joint_stop:
 * [n_ctrl_steps][nj_total], NaN keeps a joint's own stops); replaces the
 * dJointSetHingeParam / dJointSetHinge2Param(dParamLoStop, dParamHiStop)
 * calls made before each step. NULL removes them. */
int odegpuBatchSetJointStops(odegpuBatchID b, int n_ctrl_steps, const double* stops);
/* Index of the next step (selects the control row step % n_ctrl_steps); it
 * advances by one per step taken. */
int odegpuBatchSetStepIndex(odegpuBatchID b, int step);

/* Parity taps: run ONE step and copy out, per world in ODE's island/row
 * order, the rows before scaling (32 floats per row: J[12], rhs at [24],
 * cfm/h at [25], lo [26], hi [27], findex [28], b1 [29], b2 [30], joint [31],
 * as int bits for the last four), lambda after SOR, and cforce per body.
 * rows: [row_capacity][32], lambda: [row_capacity], fc: [nb_total][6]; the
 * world's rows start at row_off[w] (returned, [n_worlds]). */
int odegpuBatchStepTap(odegpuBatchID b, float* rows, float* lambda, float* fc, int* row_off);

/* Ray queries (ODE's ray geom, dRayClass). For each ray, dCollide(ray, g,
 * flags) runs on the GPU against every geom g of the ray's world
 * (ode/src/ray.cpp:196-498; a heightfield through its plane pass,
 * ode/src/heightfield.cpp:1035-1040) and the contact of least depth (the
 * distance along the ray) is kept, the lower geom index on ties: the nearest
 * hit that dSpaceCollide2(ray, space, ...) with a nearest-contact callback
 * finds (ode/src/collision_space.cpp; its bounding-box test only culls). A
 * ray attached to a body (body >= 0, world-local) skips that body's geoms as
 * dCollide does for two geoms on one body (ode/src/collision_kernel.cpp:296-303),
 * and its start and direction are in the body frame, placed with the body's
 * pose at the time of the query (a geom offset, dGeomSetOffsetPosition,
 * include/ode/collision.h:545). The direction is normalised as dGeomRaySet
 * does (ode/src/ray.cpp:115-136). flags: dCollide's, 1 to 8 contacts per
 * geom. */
typedef struct {
  int world;           /* world index */
  int body;            /* world-local body the ray is attached to, or -1 */
  float start[3];      /* world frame, or body frame when attached */
  float dir[3];        /* same frame as start */
  float length;        /* dGeomRaySetLength */
} odegpuRay;           /* 36 bytes */
typedef struct {
  int geom;            /* world-local geom index of the nearest hit; -1: no hit;
                          -2: invalid ray (world / body out of range, length
                          negative or not finite); -3: a heightfield zone under
                          the ray exceeds the lane's 10 x 10 samples (the
                          device entry only: the host entry casts such rays
                          again with workspaces of up to 128 x 128 samples) */
  float pos[3];        /* dContactGeom pos, normal, depth of dCollide(ray, geom) */
  float normal[3];
  float depth;
} odegpuRayHit;        /* 32 bytes */
/* Host arrays; returns the number of rays that hit something, or an error
 * (ODEGPU_E_ARG for an invalid ray). Runs after the batch's queued work. */
int odegpuBatchRayCast(odegpuBatchID b, const odegpuRay* rays, int n, int flags, odegpuRayHit* hits);
/* Device arrays, enqueued on the batch stream without synchronising (so it can
 * sit between steps and inside a captured graph); invalid rays come back with
 * geom = -2. */
int odegpuBatchRayCastAsync(odegpuBatchID b, const odegpuRay* d_rays, int n, int flags, odegpuRayHit* d_hits);

/* Contacts generated by the last step of world w (up to cap records of
 * pos[3] normal[3] depth b1 b2 as floats); returns the count or an error. */
int odegpuBatchGetContacts(odegpuBatchID b, int w, float* out, int cap);

/* dCollide for callers that cannot allocate device memory. It has no
 * counterpart in the reference. Hosts that own every device allocation (a
 * pool allocator they do not share, a real-time loop that forbids allocation,
 * a plugin inside a host that holds the memory budget) cannot let dCollide
 * cudaMalloc its per-call staging buffer; this entry point stages the result
 * in a fixed device array compiled into the library instead (a few hundred
 * bytes, held by every GPU that loads the library until the process exits)
 * and allocates nothing.
 *   - Geoms are given by class (ODEGPU_GEOM_SPHERE, _BOX, _CAPSULE,
 *     _CYLINDER, _PLANE or _RAY; any other class, heightfields included,
 *     fails with ODEGPU_E_ARG), class parameters as in odegpuScene
 *     (4 floats), position (3) and a 3x4 row-major rotation (12); pos/R may
 *     be NULL for a plane.
 *   - flags & 0xffff contacts are requested, at most
 *     ODEGPU_NOALLOC_MAX_CONTACTS; a larger request fails with ODEGPU_E_LIMIT.
 *   - contacts_out (host memory) receives count x 7 floats: pos[3],
 *     normal[3], depth, with dCollide's conventions; nothing past the count
 *     is written. Returns the count.
 *   - Each call, with the caller's device current, looks up the array's
 *     device address in the current context (cudaGetSymbolAddress, which
 *     allocates nothing), launches the collider on the legacy default stream
 *     and copies the contacts back synchronously before returning.
 *   - All calls share the one array; its count is reset at the start of each
 *     call, and it keeps the last call's contents afterwards. Calls from
 *     several host threads that overlap on the GPU race on it. */
#define ODEGPU_NOALLOC_MAX_CONTACTS 8
int odegpuCollideNoAlloc(int class1, const float* params1, const float* pos1, const float* R1,
                         int class2, const float* params2, const float* pos2, const float* R2,
                         int flags, float* contacts_out);

const char* odegpuGetLastError(void);

#ifdef __cplusplus
}
#endif
#endif
