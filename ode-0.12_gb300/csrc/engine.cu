// engine.cu -- batch of ODE worlds on the GPU: upload, the persistent
// warp-per-world step kernel, graph capture, state exchange and the C ABI of
// include/odegpu.h.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "odegpu.h"
#include "engine_types.cuh"
#include "world_solve.cuh"
#include "raycast.cuh"
#include "world_exact.cuh"
#include "adjoint.cuh"
#include "large_world.cuh"
#include "engine_internal.hpp"
#include "host_setup.hpp"

using namespace og;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
#define OG_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(ODEGPU_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Step = two kernels, each one warp per world; warps never wait on each other.
// `order` (optional) maps grid slots to worlds, largest worlds first, so the
// long worlds start early and the short ones fill in behind them.
__device__ __forceinline__ int slot_world(const int* order, int first, int count, int nw) {
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= count) return -1;
  const int w = order ? order[first + i] : first + i;
  return w < nw ? w : -1;
}

__global__ void __launch_bounds__(128, 4) world_collide_kernel(BatchDev d, const int* order, int first, int count,
                                                            int step, StepOptions opt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int w = slot_world(order, first, count, d.n_worlds);
  if (w < 0) return;
  if (d.world[w].nb > kMaxB || d.world[w].ng > kMaxB + 8) {
    if (lane == 0) { atomicOr(&d.status[w], ST_TOO_LARGE); d.ncontacts[w] = 0; }
    return;
  }
  const WarpSmem S = carve_collide_smem(smem_raw + (size_t)(threadIdx.x >> 5) * kCollideSmemPerWarp);
  world_collide(d, w, step, S, lane, opt);
}

__global__ void __launch_bounds__(256) world_setup_kernel(BatchDev d, const int* order, int first, int count,
                                                          int step, StepOptions opt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int w = slot_world(order, first, count, d.n_worlds);
  if (w < 0) return;
  if (d.world[w].nb > kMaxB || d.world[w].ng > kMaxB + 8) {
    if (lane == 0) { d.nrows[w] = 0; d.nislands[w] = 0; }
    return;
  }
  const WarpSmem S = carve_smem(smem_raw + (size_t)(threadIdx.x >> 5) * kSmemPerWarp);
  world_setup(d, w, step, S, lane, opt);
}

// Two register budgets of the solve kernel: world_solve_kernel keeps its
// working set in registers (168 per thread, 12 warps per SM),
// world_solve_kernel_r128 is capped at 128 for 16 warps per SM at the price of
// a few spills; batches of large worlds run faster on the first, batches of
// small ones on the second (odegpuBatchSetLaunchConfigEx / odegpuBatchAutotune
// pick).
__device__ __forceinline__ void solve_kernel_body(const BatchDev& d, const int* order, int first, int count,
                                                  const StepOptions& opt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int w = slot_world(order, first, count, d.n_worlds);
  if (w < 0) return;
  if (d.world[w].nb > kMaxB) return;
  world_solve(d, w, smem_raw + (size_t)(threadIdx.x >> 5) * kFwdSmemPerWarp, lane, opt);
}
__global__ void __launch_bounds__(256) world_solve_kernel(BatchDev d, const int* order, int first, int count,
                                                          StepOptions opt) {
  solve_kernel_body(d, order, first, count, opt);
}
__global__ void __launch_bounds__(256, 2) world_solve_kernel_r128(BatchDev d, const int* order, int first,
                                                                  int count, StepOptions opt) {
  solve_kernel_body(d, order, first, count, opt);
}

// The three phases of a step in one launch: each warp runs collide, setup and
// solve of its world back to back, handing contacts and rows over through
// global memory as the separate kernels do (program order within the warp and
// __syncwarp stand in for the kernel boundaries). Worlds do not wait for one
// another between phases, so the short worlds of a batch fill the SMs while
// the long ones are still sweeping, instead of every phase ending in a tail.
constexpr int kStepSmemPerWarp =
    kSmemPerWarp > kFwdSmemPerWarp ? (kSmemPerWarp > kCollideSmemPerWarp ? kSmemPerWarp : kCollideSmemPerWarp)
                                   : (kFwdSmemPerWarp > kCollideSmemPerWarp ? kFwdSmemPerWarp : kCollideSmemPerWarp);
__global__ void __launch_bounds__(128, 3) world_step_kernel(BatchDev d, const int* order, int first, int count,
                                                            int step, StepOptions opt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int w = slot_world(order, first, count, d.n_worlds);
  if (w < 0) return;
  unsigned char* base = smem_raw + (size_t)(threadIdx.x >> 5) * kStepSmemPerWarp;
  // the separate kernels' handling of worlds above the on-chip limits
  if (d.world[w].nb > kMaxB || d.world[w].ng > kMaxB + 8) {
    if (lane == 0) {
      atomicOr(&d.status[w], ST_TOO_LARGE);
      d.ncontacts[w] = 0;
      d.nrows[w] = 0;
      d.nislands[w] = 0;
    }
    if (d.world[w].nb > kMaxB) return;
    __syncwarp();
  } else {
    world_collide(d, w, step, carve_collide_smem(base), lane, opt);
    __syncwarp();
    world_setup(d, w, step, carve_smem(base), lane, opt);
  }
  __syncwarp();
  world_solve(d, w, base, lane, opt);
}

__global__ void __launch_bounds__(128) world_exact_kernel(BatchDev d, ExactDev X, const int* order, int first,
                                                          int count, int step, StepOptions opt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int w = slot_world(order, first, count, d.n_worlds);
  if (w < 0) return;
  if (d.world[w].nb > kMaxB || d.world[w].ng > kMaxB + 8) {
    if (lane == 0) { d.nrows[w] = 0; d.nislands[w] = 0; }
    return;
  }
  const WarpSmem S = carve_smem(smem_raw + (size_t)(threadIdx.x >> 5) * kSmemPerWarp);
  world_exact(d, X, w, step, S, lane, opt);
}
constexpr int kExactWarps = 4;

// State exchange: FP32 records of 13 floats per body.
__global__ void pack_state_kernel(BatchDev d, int nb, float* out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const float4 p = d.pos[b], q = d.q[b], v = d.lvel[b], w = d.avel[b];
  float* o = out + (size_t)b * ODEGPU_BODY_REC;
  o[0] = p.x; o[1] = p.y; o[2] = p.z;
  o[3] = q.x; o[4] = q.y; o[5] = q.z; o[6] = q.w;
  o[7] = v.x; o[8] = v.y; o[9] = v.z;
  o[10] = w.x; o[11] = w.y; o[12] = w.z;
}
__global__ void unpack_state_kernel(BatchDev d, int nb, const float* in) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const float* o = in + (size_t)b * ODEGPU_BODY_REC;
  d.pos[b] = make_float4(o[0], o[1], o[2], 0.f);
  d.q[b] = make_float4(o[3], o[4], o[5], o[6]);
  d.lvel[b] = make_float4(o[7], o[8], o[9], 0.f);
  d.avel[b] = make_float4(o[10], o[11], o[12], 0.f);
}

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DBuf() { if (p) cudaFree(p); }
  int alloc(size_t count) {
    n = count;
    if (count == 0) count = 1;
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return fail(ODEGPU_E_NOMEM, "cudaMalloc failed for " + std::to_string(count * sizeof(T)) + " bytes");
    }
    return 0;
  }
  int upload(const std::vector<T>& v) {
    if (int rc = alloc(v.size())) return rc;
    if (!v.empty() && cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(ODEGPU_E_CUDA, "upload failed");
    return 0;
  }
};

// Buffers of the large-world pipeline (large_world.cuh), sized at creation.
struct LargeWorld {
  LWDev L{};
  DBuf<int> statics, ghash, hcount, hfill, hgeoms, plist, pcnt, own, sflag, pair_i, pair_k, npairs, pnc;
  DBuf<Contact> staged;
  DBuf<int> ccount, acount, afill, adj_joint, adj_other, jentry, jlist, istart, nj, stack;
  DBuf<unsigned char> bflag;
  DBuf<int> jm, bfk, rstart;
  DBuf<float> tmp1;
  DBuf<int> rowisl, neg, draws, order, order2, rnd, tcount, tfill, tlist, bcount, bfill, blist;
  DBuf<int4> prec;
  DBuf<int> plev, lorder;
  DBuf<int2> ppred;
  DBuf<float> rsort;
  DBuf<float> lambda, fc;
  DBuf<int> err;
  DBuf<unsigned long long> stats;
  int sweep_smem = 0, islands_smem = 0;
};

constexpr int kLwIslandsSmem = 227 * 1024;

}  // namespace

struct odegpuBatch {
  int device = 0;
  int n_worlds = 0, nb_total = 0, ng_total = 0, nj_total = 0;
  long long row_cap_total = 0, contact_cap_total = 0;
  int warps_per_block = 4;
  // per-kernel launch shape: warps per block and preferred shared-memory
  // carveout (percent of the unified L1/shared array, -1 = driver default)
  // for the collide, setup, solve, adjoint and fused step kernels
  // (odegpuBatchSetLaunchConfig / odegpuBatchAutotune)
  int kwpb[5] = {4, 4, 4, 4, 4};
  int kcarve[5] = {-1, -1, -1, -1, -1};
  // a step is one world_step_kernel launch (fused) or the collide, setup and
  // solve kernels (odegpuBatchSetStepKernels / odegpuBatchAutotune)
  bool fused = false;
  // the solve kernel's register budget: 168 (false) or 128 (true) per thread
  bool solve_lowreg = false;
  int step_counter = 0;
  cudaStream_t stream = nullptr;
  std::vector<WorldDesc> h_world;

  DBuf<WorldDesc> world;
  DBuf<unsigned> seed;
  DBuf<int> status, ncontacts, nrows, nislands;
  DBuf<float4> pos, q, lvel, avel, facc, tacc;
  DBuf<float> mass, invMass, I, invI, invIw;
  DBuf<int> bflags;
  DBuf<float4> bstep;          // dxStepBody options (kStepRec per body)
  bool bstep_on = false;       // some body uses one
  DBuf<int> gtype, gbody, gsurf;
  DBuf<float4> gparam, gpos;
  DBuf<float> gbound;
  DBuf<DevHeightfield> hfs;
  DBuf<float> hf_heights;
  DBuf<DevSurface> surfaces;
  DBuf<DevJoint> joints;
  DBuf<int> padj_start, padj;
  DBuf<float> joint_torque, body_force, joint_stop;
  int n_ctrl_steps = 0;
  DBuf<DevContact> contacts;
  DBuf<float> rows;
  DBuf<float4> sweep;                // forward sweep buffers (sor_fwd.cuh)
  DBuf<unsigned char> fwd_scratch;
  DBuf<unsigned char> hf_ws;          // heightfield zone workspaces (WorldDesc::hf_ws)
  DBuf<int> jlist, adj, adj_start, island_jstart, island_rstart, jrow, jm;
  DBuf<float> state_scratch;
  DBuf<odegpuRay> ray_in;          // odegpuBatchRayCast staging, grown on demand
  DBuf<odegpuRayHit> ray_out;
  DBuf<unsigned char> ray_ws;      // heightfield workspaces of the second ray pass
  DBuf<int> ray_list;              // rays of the second pass
  double hf_min_spacing = 0.0;     // finest sample spacing of the batch's heightfields (0: none)
  bool exact = false;              // dWorldStep instead of dWorldQuickStep
  // dWorldStep scratch (world_exact.cuh). A step outside a graph sizes each
  // world's region by the rows its joints and this step's contacts can need
  // (exact_size_kernel), reads the total back and grows the arena to fit.
  // A graph cannot read anything back, so capturing dWorldStep first lays
  // the arena out by every world's row capacity (xoff_cap / xcap_cap).
  DBuf<float> xscratch;
  DBuf<long long> xoff, xoff_cap, xtotal;
  DBuf<int> xcap, xcap_cap;
  long long* xtotal_h = nullptr;     // pinned
  bool xcap_ready = false;
  int grow_exact_arena(long long floats) {
    if (xscratch.p && (long long)xscratch.n >= floats) return 0;
    if (xscratch.p) { cudaFree(xscratch.p); xscratch.p = nullptr; }
    return xscratch.alloc((size_t)(floats + floats / 4));
  }
  int ensure_exact_by_capacity() {
    if (xcap_ready) return grow_exact_arena(xtotal_cap);
    std::vector<long long> off(n_worlds);
    std::vector<int> cap(n_worlds);
    long long total = 0;
    for (int w = 0; w < n_worlds; ++w) {
      cap[w] = std::max(1, std::min(h_world[w].row_cap, kMaxR));
      off[w] = total;
      total += (exact_scratch_floats(cap[w]) + 3) & ~3LL;
    }
    if (int rc = xoff_cap.upload(off)) return rc;
    if (int rc = xcap_cap.upload(cap)) return rc;
    xtotal_cap = total;
    xcap_ready = true;
    return grow_exact_arena(total);
  }
  long long xtotal_cap = 0;
  int size_exact_step() {
    if (!xoff.p) {
      if (int rc = xoff.alloc(n_worlds)) return rc;
      if (int rc = xcap.alloc(n_worlds)) return rc;
      if (int rc = xtotal.alloc(1)) return rc;
    }
    if (!xtotal_h && cudaHostAlloc(&xtotal_h, sizeof(long long), cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      xtotal_h = nullptr;
      return fail(ODEGPU_E_NOMEM, "pinned host allocation failed");
    }
    exact_size_kernel<<<1, kExactSizeThreads, 0, stream>>>(dev(), xcap.p, xoff.p, xtotal.p);
    ++launches;
    OG_CUDA(cudaMemcpyAsync(xtotal_h, xtotal.p, sizeof(long long), cudaMemcpyDeviceToHost, stream));
    OG_CUDA(cudaStreamSynchronize(stream));
    return grow_exact_arena(*xtotal_h);
  }

  BatchDev dev() const {
    BatchDev d;
    d.n_worlds = n_worlds;
    d.world = world.p;
    d.seed = seed.p; d.status = status.p; d.ncontacts = ncontacts.p; d.nrows = nrows.p;
    d.nislands = nislands.p;
    d.pos = pos.p; d.q = q.p; d.lvel = lvel.p; d.avel = avel.p;
    d.mass = mass.p; d.invMass = invMass.p; d.I = I.p; d.invI = invI.p; d.bflags = bflags.p;
    d.bstep = bstep_on ? bstep.p : nullptr;
    d.invIw = invIw.p; d.facc = facc.p; d.tacc = tacc.p;
    d.gtype = gtype.p; d.gbody = gbody.p; d.gparam = gparam.p; d.gbound = gbound.p; d.gpos = gpos.p;
    d.gsurf = gsurf.p; d.surfaces = surfaces.p;
    d.hfs = hfs.p; d.hf_heights = hf_heights.p;
    d.joints = joints.p; d.padj_start = padj_start.p; d.padj = padj.p;
    d.n_ctrl_steps = n_ctrl_steps;
    d.joint_torque = n_ctrl_steps > 0 ? joint_torque.p : nullptr;
    d.body_force = n_ctrl_steps > 0 ? body_force.p : nullptr;
    d.joint_stop = n_ctrl_steps > 0 ? joint_stop.p : nullptr;
    d.step_counter_base = 0;
    d.contacts = contacts.p; d.rows = rows.p; d.sweep = sweep.p; d.fwd_scratch = fwd_scratch.p;
    d.hf_ws = hf_ws.p;
    d.jlist = jlist.p; d.adj = adj.p;
    d.adj_start = adj_start.p; d.island_jstart = island_jstart.p; d.island_rstart = island_rstart.p;
    d.jrow = jrow.p; d.jm = jm.p;
    return d;
  }

  DBuf<int> order;   // worlds by decreasing size (launch slot -> world)
  LargeWorld* lw = nullptr;           // set when the batch is one world above the on-chip limits

  long long launches = 0;             // kernels launched by this batch
  // Optional per-kernel timing: 4 events per step on the batch stream
  // (before collide, after collide, after setup, after solve).
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  cudaEvent_t next_event() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }
  void mark(bool on) {
    if (!on) return;
    if (cudaEvent_t e = next_event()) cudaEventRecord(e, stream);
  }
  ~odegpuBatch() {
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
    if (xtotal_h) cudaFreeHost(xtotal_h);
    delete lw;
  }

  // Rollout record for the adjoint: state and RNG seeds every `ckpt` steps
  // from step `start`, plus the state at the end.
  struct Rollout {
    int n_steps = 0, ckpt = 0, start = 0, valid = 0;
    DBuf<float> ckpt_state, seg_state, final_state;
    DBuf<unsigned> ckpt_seed, seg_seed, final_seed;
    DBuf<float> state_bar, body_tmp, row_tmp, lam_tape, dbg;
    DBuf<unsigned char> code_tape;
    DBuf<uint16_t> seq_tape;
    DBuf<int> status;
    int iters_max = 0, rounds_max = 0;
  } ro;

  int pack_to(float* out) {
    pack_state_kernel<<<(nb_total + 255) / 256, 256, 0, stream>>>(dev(), nb_total, out);
    launches += 1;
    return 0;
  }
  int unpack_from(const float* in) {
    unpack_state_kernel<<<(nb_total + 255) / 256, 256, 0, stream>>>(dev(), nb_total, in);
    launches += 1;
    return 0;
  }
  // collide + setup of one step of every world (no solve), for the adjoint
  int launch_setup(int step, const StepOptions& opt) {
    const BatchDev d = dev();
    apply_carveout(0);
    world_collide_kernel<<<nblocks(n_worlds, 0), kwpb[0] * 32, (size_t)kwpb[0] * kCollideSmemPerWarp, stream>>>(
        d, order.p, 0, n_worlds, step, opt);
    apply_carveout(1);
    world_setup_kernel<<<nblocks(n_worlds, 1), kwpb[1] * 32, (size_t)kwpb[1] * kSmemPerWarp, stream>>>(
        d, order.p, 0, n_worlds, step, opt);
    launches += 2;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ODEGPU_E_CUDA, std::string("setup launch: ") + cudaGetErrorString(e));
    return 0;
  }

  // n_steps steps of worlds [first, first+count) of the launch order (or of
  // the identity order when use_order is false); 3 launches per step.
  DBuf<float> jcopy, feedback;       // joint feedback (odegpuBatchSetFeedback)
  bool feedback_on = false;
  bool single_world = false;         // one world per launch (the plain comparator)

  int nblocks(int count, int k) const { return (count + kwpb[k] - 1) / kwpb[k]; }
  // the carveout is a property of the kernel function: set it when it differs
  // from what the last launch of that kernel used (any batch)
  void apply_carveout(int k) {
    static int current[6] = {-1, -1, -1, -1, -1, -1};   // slot 5: the 128-register solve kernel
    const int slot = (k == 2 && solve_lowreg) ? 5 : k;
    if (current[slot] == kcarve[k]) return;
    const void* fn = k == 0 ? (const void*)world_collide_kernel
                   : k == 1 ? (const void*)world_setup_kernel
                   : k == 2 ? (solve_lowreg ? (const void*)world_solve_kernel_r128 : (const void*)world_solve_kernel)
                   : k == 3 ? (const void*)adjoint_step_kernel : (const void*)world_step_kernel;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, kcarve[k]) == cudaSuccess)
      current[slot] = kcarve[k];
    else
      cudaGetLastError();
  }

  // Steps of the large world (large_world.cuh): ~30 launches plus ~11 per
  // reshuffle round, all on the batch stream (capturable into a graph).
  int lw_launch(int n_steps, const StepOptions& opt) {
    LargeWorld& W = *lw;
    const BatchDev d = dev();
    const WorldDesc& D = h_world[0];
    const LWDev L0 = W.L;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(stream, &cap);
    const bool tm = timing && cap == cudaStreamCaptureStatusNone;
    auto g = [](long long n, int t) { return (unsigned)std::max(1LL, (n + t - 1) / t); };
    const int T = 256;
    const int nb = L0.nb, ng = L0.ng, njall = L0.njp + L0.contact_cap, R = L0.row_cap;
    auto scan = [&](int* a, const int* n_dev, int n_host, int rows = 1, size_t stride = 0) {
      lw_scan_kernel<<<rows, kLwScanThreads, 0, stream>>>(a, n_dev, n_host, stride);
      ++launches;
    };
    const bool joint_ctl = !opt.host_forces && n_ctrl_steps > 0 && joint_torque.p && D.njp > 0;
    for (int s = 0; s < n_steps; ++s) {
      const int step = step_counter + s;
      mark(tm);
      cudaMemsetAsync(L0.err, 0, sizeof(int), stream);
      if (joint_ctl) {
        lw_bodies_pre_kernel<<<g(nb, T), T, 0, stream>>>(d, step, 1, 0);
        lw_controls_joints_kernel<<<1, 32, 0, stream>>>(d, step);
        lw_bodies_pre_kernel<<<g(nb, T), T, 0, stream>>>(d, step, 0, 1);
        launches += 3;
      } else {
        lw_bodies_pre_kernel<<<g(nb, T), T, 0, stream>>>(d, step, opt.host_forces ? 0 : 1, 1);
        launches += 1;
      }
      cudaMemsetAsync(L0.ccount, 0, sizeof(int) * nb, stream);
      cudaMemsetAsync(L0.afill, 0, sizeof(int) * nb, stream);
      if (opt.collide) {
        // broadphase + narrowphase in canonical pair order
        cudaMemsetAsync(L0.hcount, 0, sizeof(int) * (L0.hsize + 1), stream);
        cudaMemsetAsync(L0.hfill, 0, sizeof(int) * L0.hsize, stream);
        if (L0.nstat) cudaMemsetAsync(L0.sflag, 0, sizeof(int) * (size_t)L0.nstat * (ng + 1), stream);
        lw_hash_kernel<<<g(ng, T), T, 0, stream>>>(d, L0);
        scan(L0.hcount, nullptr, L0.hsize);
        lw_hfill_kernel<<<g(ng, T), T, 0, stream>>>(L0);
        lw_candidates_kernel<<<g(ng, 128), 128, 0, stream>>>(d, L0);
        launches += 3;
        if (L0.nstat) {
          scan(L0.sflag, nullptr, ng, L0.nstat, (size_t)ng + 1);
          lw_static_own_kernel<<<1, 32, 0, stream>>>(L0);
          ++launches;
        }
        scan(L0.own, nullptr, ng);
        lw_pairs_fill_kernel<<<g(ng, T), T, 0, stream>>>(d, L0);
        lw_narrow_kernel<<<g(L0.pair_cap, 128), 128, 0, stream>>>(d, L0);
        if (D.hf_ws_side > 0) {
          lw_hf_big_kernel<<<1, 32, 0, stream>>>(d, L0);
          ++launches;
        }
        scan(L0.pnc, L0.npairs, 0);
        lw_contacts_kernel<<<g(L0.pair_cap, T), T, 0, stream>>>(d, L0);
        launches += 3;
      }
      mark(tm);
      // body joint lists (contacts newest first, then persistent joints; or
      // the host's complete lists), islands, rows
      lw_adj_count_kernel<<<g(nb, T), T, 0, stream>>>(d, L0);
      scan(L0.acount, nullptr, nb);
      if (!opt.host_adjacency) {
        lw_adj_fill_kernel<<<g(L0.contact_cap, T), T, 0, stream>>>(d, L0);
        ++launches;
      }
      lw_adj_finish_kernel<<<g(nb, T), T, 0, stream>>>(d, L0);
      lw_islands_kernel<<<1, 32, W.islands_smem, stream>>>(d, L0, W.islands_smem);
      lw_info1_kernel<<<g(njall, 128), 128, 0, stream>>>(d, L0, step);
      launches += 4;
      scan(L0.jm, L0.nj, 0);
      lw_max_scan_kernel<<<1, kLwScanThreads, 0, stream>>>(L0.bfk, L0.nj);
      lw_info2_kernel<<<g(njall, 128), 128, 0, stream>>>(d, L0, step);
      lw_tmp1_kernel<<<g(nb, T), T, 0, stream>>>(d, L0);
      const bool fb = opt.jcopy && (opt.feedback || opt.contact_feedback);
      lw_row_setup_kernel<<<g(R, T), T, 0, stream>>>(d, L0, fb ? opt.jcopy : nullptr);
      launches += 4;
      mark(tm);
      // SOR: initial order, then per reshuffle round the exact permutation,
      // the per-body ranks and the cluster sweep of up to 8 iterations
      lw_order_flags_kernel<<<g(std::max(R, nb), T), T, 0, stream>>>(d, L0);
      ++launches;
      scan(L0.neg, d.nrows, 0);
      scan(L0.draws, d.nislands, 0);
      lw_order_init_kernel<<<g(R, T), T, 0, stream>>>(d, L0);
      ++launches;
      int* cur = L0.order;
      int* nxt = L0.order2;
      const int iters = D.iterations;
      for (int round = 0; round * 8 < iters; ++round) {
        cudaMemsetAsync(L0.tcount, 0, sizeof(int) * (R + 1), stream);
        cudaMemsetAsync(L0.tfill, 0, sizeof(int) * R, stream);
        cudaMemsetAsync(L0.bcount, 0, sizeof(int) * (nb + 1), stream);
        cudaMemsetAsync(L0.bfill, 0, sizeof(int) * nb, stream);
        lw_rand_kernel<<<g(R, T), T, 0, stream>>>(d, L0, round);
        scan(L0.tcount, d.nrows, 0);
        lw_tfill_kernel<<<g(R, T), T, 0, stream>>>(d, L0);
        lw_tsort_kernel<<<g(R, T), T, 0, stream>>>(d, L0);
        lw_permute_kernel<<<g(R, T), T, 0, stream>>>(d, L0, cur, nxt);
        std::swap(cur, nxt);
        lw_bodypos_kernel<<<g(R, T), T, 0, stream>>>(d, L0, cur);
        scan(L0.bcount, nullptr, nb);
        lw_bfill_kernel<<<g(R, T), T, 0, stream>>>(d, L0, cur);
        lw_branks_kernel<<<g(nb, T), T, 0, stream>>>(d, L0, cur);
        launches += 7;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)L0.cluster);
        cfg.blockDim = dim3(kLwSweepThreads);
        cfg.dynamicSmemBytes = (size_t)W.sweep_smem;
        cfg.stream = stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)L0.cluster;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        const int it1 = std::min(iters, 8 * round + 8);
        cudaError_t e = cudaLaunchKernelEx(&cfg, lw_sweep_kernel, d, L0, 8 * round, it1, round == 0 ? 1 : 0);
        if (e != cudaSuccess) return fail(ODEGPU_E_CUDA, std::string("sweep launch: ") + cudaGetErrorString(e));
        ++launches;
      }
      if (fb) {
        lw_feedback_kernel<<<g(njall, 128), 128, 0, stream>>>(d, L0, opt.jcopy, opt.feedback, opt.contact_feedback);
        ++launches;
      }
      lw_integrate_kernel<<<g(nb, T), T, 0, stream>>>(d, L0);
      ++launches;
      mark(tm);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ODEGPU_E_CUDA, std::string("large-world step: ") + cudaGetErrorString(e));
    return 0;
  }

  int launch(int first, int count, int n_steps, const StepOptions& opt_in, bool use_order = true) {
    StepOptions opt = opt_in;
    if (feedback_on) { opt.jcopy = jcopy.p; opt.feedback = feedback.p; }
    if (lw) return lw_launch(n_steps, opt);
    const BatchDev d = dev();
    const int* ord = (use_order && order.p) ? order.p : nullptr;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(stream, &cap);
    const bool tm = timing && cap == cudaStreamCaptureStatusNone;
    int w[3];
    for (int k = 0; k < 3; ++k) w[k] = single_world ? 1 : kwpb[k];
    if (exact) {
      const bool capturing = cap != cudaStreamCaptureStatusNone;
      if (capturing && !(xcap_ready && xscratch.p && (long long)xscratch.n >= xtotal_cap))
        return fail(ODEGPU_E_ARG, "dWorldStep scratch was not laid out before the capture");
      const int wx = single_world ? 1 : kExactWarps;
      for (int s = 0; s < n_steps; ++s) {
        mark(tm);
        apply_carveout(0);
        world_collide_kernel<<<(count + w[0] - 1) / w[0], w[0] * 32, (size_t)w[0] * kCollideSmemPerWarp,
                               stream>>>(d, ord, first, count, step_counter + s, opt);
        if (!capturing)
          if (int rc = size_exact_step()) return rc;
        const ExactDev X = capturing ? ExactDev{xscratch.p, xoff_cap.p, xcap_cap.p}
                                     : ExactDev{xscratch.p, xoff.p, xcap.p};
        mark(tm);
        world_exact_kernel<<<(count + wx - 1) / wx, wx * 32, (size_t)wx * kSmemPerWarp, stream>>>(
            d, X, ord, first, count, step_counter + s, opt);
        mark(tm);
        mark(tm);
        launches += 2;
      }
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return fail(ODEGPU_E_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
      return 0;
    }
    if (fused) {
      // one launch per step; with timing on, its time is recorded in the
      // collide slot and the setup and solve slots stay empty
      const int wf = single_world ? 1 : kwpb[4];
      for (int s = 0; s < n_steps; ++s) {
        mark(tm);
        apply_carveout(4);
        world_step_kernel<<<(count + wf - 1) / wf, wf * 32, (size_t)wf * kStepSmemPerWarp, stream>>>(
            d, ord, first, count, step_counter + s, opt);
        mark(tm);
        mark(tm);
        mark(tm);
        launches += 1;
      }
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return fail(ODEGPU_E_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
      return 0;
    }
    for (int s = 0; s < n_steps; ++s) {
      mark(tm);
      apply_carveout(0);
      world_collide_kernel<<<(count + w[0] - 1) / w[0], w[0] * 32, (size_t)w[0] * kCollideSmemPerWarp, stream>>>(
          d, ord, first, count, step_counter + s, opt);
      mark(tm);
      apply_carveout(1);
      world_setup_kernel<<<(count + w[1] - 1) / w[1], w[1] * 32, (size_t)w[1] * kSmemPerWarp, stream>>>(
          d, ord, first, count, step_counter + s, opt);
      mark(tm);
      apply_carveout(2);
      if (solve_lowreg)
        world_solve_kernel_r128<<<(count + w[2] - 1) / w[2], w[2] * 32, (size_t)w[2] * kFwdSmemPerWarp, stream>>>(
            d, ord, first, count, opt);
      else
        world_solve_kernel<<<(count + w[2] - 1) / w[2], w[2] * 32, (size_t)w[2] * kFwdSmemPerWarp, stream>>>(
            d, ord, first, count, opt);
      mark(tm);
      launches += 3;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ODEGPU_E_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
    return 0;
  }
};

// Largest block shapes (warps per block) the launch configuration accepts.
constexpr int kMaxWpb[5] = {4, 8, 8, 4, 4};

static int configure_kernels() {
  if (cudaFuncSetAttribute(world_collide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(kMaxWpb[0] * kCollideSmemPerWarp)) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(world_setup_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(kMaxWpb[1] * kSmemPerWarp)) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(world_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(kMaxWpb[2] * kFwdSmemPerWarp)) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(world_solve_kernel_r128, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(kMaxWpb[2] * kFwdSmemPerWarp)) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(adjoint_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(kMaxWpb[3] * kAdjSmemPerWarp)) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(world_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(kMaxWpb[4] * kStepSmemPerWarp)) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(world_exact_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(kExactWarps * kSmemPerWarp)) != cudaSuccess)
    return -1;
  return 0;
}

extern "C" {

const char* odegpuGetLastError(void) { return g_last_error.c_str(); }

static float bound_radius(int type, const double* p) {
  switch (type) {
    case ODEGPU_GEOM_SPHERE: return (float)p[0];
    case ODEGPU_GEOM_BOX: return (float)(0.5 * std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]));
    case ODEGPU_GEOM_CAPSULE: return (float)(p[0] + 0.5 * p[1]);
    case ODEGPU_GEOM_CYLINDER: return (float)std::sqrt(p[0] * p[0] + 0.25 * p[1] * p[1]);
    default: return INFINITY;
  }
}

// Half-extent bound, under any rotation, of the axis-aligned box that the
// reference computes for a geom (computeAABB: sphere.cpp:59-67, box.cpp:60-78,
// capsule.cpp:60-74, cylinder.cpp:58-73, ray.cpp:56-89): sizes the
// heightfield zones a geom can cover.
static double aabb_half_bound(int type, const double* p) {
  switch (type) {
    case ODEGPU_GEOM_RAY: return 0.5 * p[0];
    case ODEGPU_GEOM_SPHERE: return p[0];
    case ODEGPU_GEOM_BOX: return 0.5 * std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    case ODEGPU_GEOM_CAPSULE: return p[0] + 0.5 * p[1];
    case ODEGPU_GEOM_CYLINDER: return std::sqrt(2.0 * p[0] * p[0] + 0.25 * p[1] * p[1]);
    default: return 0.0;
  }
}
// Samples per axis of the largest zone under a geom of that bound on a field
// of sample spacing s: the floor and ceiling of the box's ends over the
// spacing, each widened by one ulp (heightfield.cpp:1742-1760), plus one.
static int hf_zone_side(double half, double s) { return (int)std::floor(2.0 * half / s + 3.0) + 1; }

static int set_joint_stops(odegpuBatch* B, int n_ctrl, const double* js) {
  if (B->joint_stop.p) { cudaFree(B->joint_stop.p); B->joint_stop.p = nullptr; }
  if (!js || n_ctrl <= 0) return 0;
  std::vector<float> v((size_t)n_ctrl * B->nj_total);
  for (size_t i = 0; i < v.size(); ++i) v[i] = (float)js[i];
  return B->joint_stop.upload(v);
}

static int set_controls(odegpuBatch* B, int n_ctrl, const double* jt, const double* bf) {
  B->n_ctrl_steps = n_ctrl;
  if (n_ctrl <= 0) { B->n_ctrl_steps = 0; return 0; }
  std::vector<float> t, f;
  if (jt) {
    t.resize((size_t)n_ctrl * B->nj_total * 2);
    for (size_t i = 0; i < t.size(); ++i) t[i] = (float)jt[i];
  }
  if (bf) {
    f.resize((size_t)n_ctrl * B->nb_total * 6);
    for (size_t i = 0; i < f.size(); ++i) f[i] = (float)bf[i];
  }
  if (B->joint_torque.p) { cudaFree(B->joint_torque.p); B->joint_torque.p = nullptr; }
  if (B->body_force.p) { cudaFree(B->body_force.p); B->body_force.p = nullptr; }
  if (jt) { if (int rc = B->joint_torque.upload(t)) return rc; }
  if (bf) { if (int rc = B->body_force.upload(f)) return rc; }
  return 0;
}

// Buffers and launch shapes of the large-world pipeline for the batch's only world.
static int lw_setup(odegpuBatch* B, const odegpuScene* sc) {
  LargeWorld& W = *B->lw;
  const WorldDesc& D = B->h_world[0];
  LWDev& L = W.L;
  L.nb = D.nb; L.ng = D.ng; L.njp = D.njp;
  L.contact_cap = D.contact_cap;
  L.row_cap = D.row_cap;
  L.pair_cap = 16 * D.ng + 1024;
  L.adj_cap = 2 * (D.njp + D.contact_cap);
  int hs = 1024;
  while (hs < 2 * D.ng) hs <<= 1;
  L.hsize = hs;
  // grid cell: at least the widest pair pre-test between two geoms on bodies
  double rmax = 0;
  std::vector<int> st;
  for (int g = 0; g < D.ng; ++g) {
    const int gg = D.geom_off + g;
    if (sc->geom_body[gg] < 0) { st.push_back(g); continue; }
    rmax = std::max(rmax, (double)bound_radius(sc->geom_type[gg], sc->geom_param + ODEGPU_GEOM_NPARAM * (size_t)gg));
  }
  const double cell = rmax > 0 ? 1.01 * (2.0 * rmax * 1.001 + 1e-5) : 1.0;
  L.cell = (float)cell;
  L.inv_cell = (float)(1.0 / cell);
  L.nstat = (int)st.size();
  const int nb = D.nb, ng = D.ng, R = D.row_cap, njall = D.njp + D.contact_cap;
  int rc = 0;
  rc = rc ? rc : W.statics.upload(st.empty() ? std::vector<int>{0} : st);
  rc = rc ? rc : W.ghash.alloc(ng);
  rc = rc ? rc : W.hcount.alloc((size_t)hs + 1);
  rc = rc ? rc : W.hfill.alloc(hs);
  rc = rc ? rc : W.hgeoms.alloc(ng);
  rc = rc ? rc : W.plist.alloc((size_t)ng * kLwPartners);
  rc = rc ? rc : W.pcnt.alloc(ng);
  rc = rc ? rc : W.own.alloc((size_t)ng + 1);
  rc = rc ? rc : W.sflag.alloc((size_t)std::max(1, L.nstat) * (ng + 1));
  rc = rc ? rc : W.pair_i.alloc(L.pair_cap);
  rc = rc ? rc : W.pair_k.alloc(L.pair_cap);
  rc = rc ? rc : W.npairs.alloc(1);
  rc = rc ? rc : W.pnc.alloc((size_t)L.pair_cap + 1);
  rc = rc ? rc : W.staged.alloc((size_t)L.pair_cap * D.max_contacts);
  rc = rc ? rc : W.ccount.alloc(nb);
  rc = rc ? rc : W.acount.alloc((size_t)nb + 1);
  rc = rc ? rc : W.afill.alloc(nb);
  rc = rc ? rc : W.adj_joint.alloc(L.adj_cap);
  rc = rc ? rc : W.adj_other.alloc(L.adj_cap);
  rc = rc ? rc : W.jentry.alloc(njall);
  rc = rc ? rc : W.jlist.alloc(njall);
  rc = rc ? rc : W.istart.alloc((size_t)nb + 1);
  rc = rc ? rc : W.nj.alloc(1);
  rc = rc ? rc : W.stack.alloc(nb);
  rc = rc ? rc : W.bflag.alloc(nb);
  rc = rc ? rc : W.jm.alloc((size_t)njall + 1);
  rc = rc ? rc : W.bfk.alloc(njall);
  rc = rc ? rc : W.rstart.alloc((size_t)nb + 1);
  rc = rc ? rc : W.tmp1.alloc((size_t)nb * 6);
  rc = rc ? rc : W.rowisl.alloc(R);
  rc = rc ? rc : W.neg.alloc((size_t)R + 1);
  rc = rc ? rc : W.draws.alloc((size_t)nb + 1);
  rc = rc ? rc : W.order.alloc(R);
  rc = rc ? rc : W.order2.alloc(R);
  rc = rc ? rc : W.rnd.alloc(R);
  rc = rc ? rc : W.tcount.alloc((size_t)R + 1);
  rc = rc ? rc : W.tfill.alloc(R);
  rc = rc ? rc : W.tlist.alloc(R);
  rc = rc ? rc : W.bcount.alloc((size_t)nb + 1);
  rc = rc ? rc : W.bfill.alloc(nb);
  rc = rc ? rc : W.blist.alloc(2 * (size_t)R);
  rc = rc ? rc : W.prec.alloc(R);
  rc = rc ? rc : W.plev.alloc(R);
  rc = rc ? rc : W.lorder.alloc(R);
  rc = rc ? rc : W.ppred.alloc(R);
  rc = rc ? rc : W.rsort.alloc((size_t)R * kRowWords);
  rc = rc ? rc : W.lambda.alloc(R);
  rc = rc ? rc : W.fc.alloc((size_t)nb * 6);
  rc = rc ? rc : W.err.alloc(1);
  rc = rc ? rc : W.stats.alloc(9);
  if (rc) return rc;
  OG_CUDA(cudaMemset(W.stats.p, 0, 9 * sizeof(unsigned long long)));
  L.statics = W.statics.p; L.ghash = W.ghash.p; L.hcount = W.hcount.p; L.hfill = W.hfill.p;
  L.hgeoms = W.hgeoms.p; L.plist = W.plist.p; L.pcnt = W.pcnt.p; L.own = W.own.p; L.sflag = W.sflag.p;
  L.pair_i = W.pair_i.p; L.pair_k = W.pair_k.p; L.npairs = W.npairs.p; L.pnc = W.pnc.p;
  L.staged = W.staged.p; L.ccount = W.ccount.p; L.acount = W.acount.p; L.afill = W.afill.p;
  L.adj_joint = W.adj_joint.p; L.adj_other = W.adj_other.p; L.jentry = W.jentry.p; L.jlist = W.jlist.p;
  L.istart = W.istart.p; L.nj = W.nj.p; L.stack = W.stack.p; L.bflag = W.bflag.p; L.jm = W.jm.p;
  L.bfk = W.bfk.p; L.rstart = W.rstart.p; L.tmp1 = W.tmp1.p; L.rowisl = W.rowisl.p; L.neg = W.neg.p;
  L.draws = W.draws.p; L.order = W.order.p; L.order2 = W.order2.p; L.rnd = W.rnd.p;
  L.tcount = W.tcount.p; L.tfill = W.tfill.p; L.tlist = W.tlist.p; L.bcount = W.bcount.p;
  L.bfill = W.bfill.p; L.blist = W.blist.p; L.prec = W.prec.p; L.plev = W.plev.p; L.lorder = W.lorder.p; L.ppred = W.ppred.p; L.rsort = W.rsort.p; L.lambda = W.lambda.p; L.fc = W.fc.p;
  L.err = W.err.p;
  L.stats = W.stats.p;
  int optin = 0;
  OG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, B->device));
  const int smem_max = std::min(optin, kLwIslandsSmem);
  OG_CUDA(cudaFuncSetAttribute(lw_islands_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
  W.islands_smem = smem_max;
  // the sweep cluster: the largest cluster (16, non-portable, down to 1) the
  // device can place with the body slots and lambdas split over its CTAs
  cudaFuncAttributes fa{};
  OG_CUDA(cudaFuncGetAttributes(&fa, lw_sweep_kernel));
  const int sweep_dyn_max = optin - (int)fa.sharedSizeBytes;
  OG_CUDA(cudaFuncSetAttribute(lw_sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sweep_dyn_max));
  cudaFuncSetAttribute(lw_sweep_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaGetLastError();
  for (int C : {16, 8, 4, 2, 1}) {
    // body slots, then per row slot a lambda and a level
    const size_t smem = (size_t)((nb + C - 1) / C) * sizeof(LwBody) + (size_t)((R + C - 1) / C) * 2 * sizeof(float);
    if (smem > (size_t)sweep_dyn_max) continue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C);
    cfg.blockDim = dim3(kLwSweepThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, (void*)lw_sweep_kernel, &cfg) == cudaSuccess && ncl >= 1) {
      L.cluster = C;
      W.sweep_smem = (int)smem;
      break;
    }
    cudaGetLastError();
  }
  if (L.cluster == 0)
    return fail(ODEGPU_E_LIMIT, "the world's bodies and rows do not fit the sweep cluster's shared memory");
  return 0;
}

int odegpuBatchCreate(const odegpuScene* sc, const odegpuBatchConfig* cfg, odegpuBatchID* out) {
  if (!sc || !out || sc->n_worlds <= 0) return fail(ODEGPU_E_ARG, "bad scene");
  *out = nullptr;
  const int dev = cfg ? cfg->device : 0;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= dev) {
    cudaGetLastError();
    return fail(ODEGPU_E_CUDA, "no CUDA device available");
  }
  OG_CUDA(cudaSetDevice(dev));
  auto* B = new odegpuBatch();
  B->device = dev;
  const int cpb = (cfg && cfg->contacts_per_body > 0) ? cfg->contacts_per_body : 8;
  B->warps_per_block = (cfg && cfg->warps_per_block > 0) ? cfg->warps_per_block : 4;
  const int W = sc->n_worlds;
  B->n_worlds = W;
  B->nb_total = sc->body_off[W];
  B->ng_total = sc->geom_off[W];
  B->nj_total = sc->joint_off[W];

  // ---- bodies (dBodySetPosition/Quaternion/Velocity, dBodySetMass)
  const int NB = B->nb_total;
  std::vector<float4> pos(NB), q(NB), lv(NB), av(NB);
  std::vector<float> mass(NB), invMass(NB), I(9 * (size_t)NB), invI(9 * (size_t)NB);
  std::vector<int> flags(NB);
  std::vector<og_host::HBody> hb(NB);
  for (int b = 0; b < NB; ++b) {
    og_host::HBody& H = hb[b];
    for (int k = 0; k < 3; ++k) H.pos[k] = sc->body_pos[3 * b + k];
    for (int k = 0; k < 4; ++k) H.q[k] = sc->body_q[4 * b + k];
    og_host::normalize4(H.q);
    og_host::r_from_q(H.R, H.q);
    pos[b] = make_float4((float)H.pos[0], (float)H.pos[1], (float)H.pos[2], 0.f);
    q[b] = make_float4((float)H.q[0], (float)H.q[1], (float)H.q[2], (float)H.q[3]);
    lv[b] = make_float4((float)sc->body_lvel[3 * b], (float)sc->body_lvel[3 * b + 1],
                        (float)sc->body_lvel[3 * b + 2], 0.f);
    av[b] = make_float4((float)sc->body_avel[3 * b], (float)sc->body_avel[3 * b + 1],
                        (float)sc->body_avel[3 * b + 2], 0.f);
    mass[b] = (float)sc->body_mass[b];
    invMass[b] = (float)(1.0 / sc->body_mass[b]);
    double inv[9];
    const double* Ib = sc->body_I + 9 * (size_t)b;
    // dMassSetParameters keeps the matrix symmetric from its upper triangle
    double Is[9] = {Ib[0], Ib[1], Ib[2], Ib[1], Ib[4], Ib[5], Ib[2], Ib[5], Ib[8]};
    if (!og_host::invert_pd3(Is, inv)) {
      for (int k = 0; k < 9; ++k) inv[k] = (k % 4 == 0) ? 1.0 : 0.0;
    }
    for (int k = 0; k < 9; ++k) { I[9 * (size_t)b + k] = (float)Is[k]; invI[9 * (size_t)b + k] = (float)inv[k]; }
    flags[b] = sc->body_flags[b];
  }

  // ---- geoms
  const int NG = B->ng_total;
  std::vector<int> gtype(NG), gbody(NG), gsurf(NG);
  std::vector<float4> gparam(NG), gpos(NG);
  std::vector<float> gbound(NG);
  for (int g = 0; g < NG; ++g) {
    gtype[g] = sc->geom_type[g];
    gbody[g] = sc->geom_body[g];
    gsurf[g] = sc->geom_surface[g];
    double p[4];
    for (int k = 0; k < 4; ++k) p[k] = sc->geom_param[ODEGPU_GEOM_NPARAM * (size_t)g + k];
    if (gtype[g] == ODEGPU_GEOM_PLANE) {
      // make_sure_plane_normal_has_unit_length (ode/src/plane.cpp:40-56)
      double l = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
      if (l > 0) { l = 1.0 / std::sqrt(l); p[0] *= l; p[1] *= l; p[2] *= l; p[3] *= l; }
      else { p[0] = 1; p[1] = p[2] = p[3] = 0; }
    } else if (gtype[g] == ODEGPU_GEOM_HEIGHTFIELD) {
      const int hi = (int)p[0];
      if (gbody[g] >= 0 || hi < 0 || hi >= sc->n_heightfields || !sc->heightfields) {
        delete B;
        return fail(ODEGPU_E_ARG, "heightfield geom: bad heightfield index or attached to a body");
      }
    } else if (gtype[g] == ODEGPU_GEOM_RAY) {
      delete B;
      return fail(ODEGPU_E_ARG, "a scene may not hold a ray geom: rays are queries (odegpuBatchRayCast)");
    } else if (gtype[g] != ODEGPU_GEOM_SPHERE && gtype[g] != ODEGPU_GEOM_BOX &&
               gtype[g] != ODEGPU_GEOM_CAPSULE && gtype[g] != ODEGPU_GEOM_CYLINDER) {
      delete B;
      return fail(ODEGPU_E_ARG, "unsupported geom class " + std::to_string(gtype[g]));
    }
    gparam[g] = make_float4((float)p[0], (float)p[1], (float)p[2], (float)p[3]);
    gpos[g] = make_float4(0.f, 0.f, 0.f, 0.f);
    gbound[g] = bound_radius(gtype[g], p);
  }
  // heightfields: dGeomHeightfieldDataBuildDouble + dxHeightfieldData::SetData
  // caches (ode/src/heightfield.cpp:107-143), samples stored as FP32
  std::vector<DevHeightfield> hfs(std::max(1, sc->n_heightfields));
  std::vector<float> hf_heights;
  for (int i = 0; i < sc->n_heightfields; ++i) {
    const odegpuHeightfield& H = sc->heightfields[i];
    if (H.nx < 2 || H.nz < 2 || !(H.width > 0) || !(H.depth > 0) || !H.heights) {
      delete B;
      return fail(ODEGPU_E_ARG, "heightfield " + std::to_string(i) + ": bad sample counts or extent");
    }
    hfs[i] = og::make_dev_heightfield(H.nx, H.nz, H.width, H.depth, H.scale, H.offset, H.thickness, H.wrap,
                                      H.pos, H.R, (int)hf_heights.size());
    for (long long k = 0; k < (long long)H.nx * H.nz; ++k) hf_heights.push_back((float)H.heights[k]);
  }
  for (int g = 0; g < NG; ++g)
    if (gtype[g] == ODEGPU_GEOM_HEIGHTFIELD) {
      const DevHeightfield& D = hfs[(int)sc->geom_param[ODEGPU_GEOM_NPARAM * (size_t)g]];
      gpos[g] = make_float4(D.pos[0], D.pos[1], D.pos[2], 0.f);
    }
  for (int i = 0; i < sc->n_heightfields; ++i) {
    const double sp = std::min(hfs[i].sw, hfs[i].sd);
    B->hf_min_spacing = B->hf_min_spacing > 0.0 ? std::min(B->hf_min_spacing, sp) : sp;
  }
  std::vector<DevSurface> surf(std::max(1, sc->n_surfaces));
  for (int s = 0; s < sc->n_surfaces; ++s) {
    const odegpuSurface& S = sc->surfaces[s];
    DevSurface& D = surf[s];
    D.mode = S.mode;
    D.mu = (float)S.mu; D.mu2 = (float)S.mu2; D.bounce = (float)S.bounce; D.bounce_vel = (float)S.bounce_vel;
    D.soft_erp = (float)S.soft_erp; D.soft_cfm = (float)S.soft_cfm; D.motion1 = (float)S.motion1;
    D.motion2 = (float)S.motion2; D.motionN = (float)S.motionN; D.slip1 = (float)S.slip1;
    D.slip2 = (float)S.slip2;
  }
  if (sc->n_surfaces <= 0) std::memset(&surf[0], 0, sizeof(DevSurface));

  // ---- worlds, joints, persistent adjacency
  std::vector<WorldDesc>& wd = B->h_world;
  wd.resize(W);
  std::vector<unsigned> seeds(W);
  std::vector<DevJoint> joints(std::max(1, B->nj_total));
  std::vector<int> padj_start((size_t)NB + W);
  std::vector<int> padj;
  long long contact_off = 0, row_off = 0, hf_ws_total = 0;
  int n_fwd_scratch = 0;
  for (int w = 0; w < W; ++w) {
    const odegpuWorldParams& P = sc->world[w];
    WorldDesc& D = wd[w];
    D.body_off = sc->body_off[w];
    D.nb = sc->body_off[w + 1] - D.body_off;
    D.geom_off = sc->geom_off[w];
    D.ng = sc->geom_off[w + 1] - D.geom_off;
    D.joint_off = sc->joint_off[w];
    D.njp = sc->joint_off[w + 1] - D.joint_off;
    if (D.nb > ODEGPU_MAX_BODIES_PER_WORLD && W > 1) {
      delete B;
      return fail(ODEGPU_E_LIMIT, "world " + std::to_string(w) + " has " + std::to_string(D.nb) +
                                      " bodies; the on-chip kernel handles at most " +
                                      std::to_string(ODEGPU_MAX_BODIES_PER_WORLD) +
                                      " (a larger world must be the only world of its batch)");
    }
    if (D.nb > ODEGPU_MAX_BODIES_LARGE) {
      delete B;
      return fail(ODEGPU_E_LIMIT, "world has " + std::to_string(D.nb) + " bodies; at most " +
                                      std::to_string(ODEGPU_MAX_BODIES_LARGE));
    }
    const bool large = W == 1 && ((cfg && cfg->large_world) || D.nb > kMaxB || D.ng > kMaxB + 8 ||
                                  D.njp + cpb * D.nb + 16 > kMaxR);
    if (P.max_contacts < 1 || P.max_contacts > 8) {
      delete B;
      return fail(ODEGPU_E_ARG, "max_contacts must be in [1, 8]");
    }
    D.contact_off = (int)contact_off;
    D.contact_cap = cpb * D.nb + 16;
    contact_off += D.contact_cap;
    D.row_off = (int)row_off;
    D.row_cap = large ? 3 * D.contact_cap + 6 * D.njp
                      : std::min(ODEGPU_MAX_ROWS_PER_WORLD, 3 * D.contact_cap + 6 * D.njp);
    if (large) B->lw = new LargeWorld();
    row_off += D.row_cap;
    D.fwd_scratch = (!large && D.row_cap > kFwdRows) ? n_fwd_scratch++ : -1;
    // a heightfield workspace for worlds whose geoms can cover more samples
    // than the lane's arrays hold
    {
      double smin = INFINITY, half = 0.0;
      for (int g = D.geom_off; g < D.geom_off + D.ng; ++g) {
        const double* gp = sc->geom_param + ODEGPU_GEOM_NPARAM * (size_t)g;
        if (gtype[g] == ODEGPU_GEOM_HEIGHTFIELD) {
          const DevHeightfield& F = hfs[(int)gp[0]];
          smin = std::min(smin, (double)std::min(F.sw, F.sd));
        } else if (gbody[g] >= 0) {
          half = std::max(half, aabb_half_bound(gtype[g], gp));
        }
      }
      D.hf_ws_side = 0;
      D.hf_ws = -1;
      if (smin < INFINITY && half > 0.0) {
        const int side = hf_zone_side(half, smin);
        if (side > kHFZone) {
          D.hf_ws_side = std::min(side, kHFBigZone);
          D.hf_ws = hf_ws_total;
          hf_ws_total += (og::hf_ws_bytes(D.hf_ws_side) + 255) & ~255LL;
        }
      }
    }
    D.max_contacts = P.max_contacts;
    D.iterations = P.iterations;
    for (int k = 0; k < 3; ++k) D.gravity[k] = (float)P.gravity[k];
    D.erp = (float)P.erp; D.cfm = (float)P.cfm; D.sor_w = (float)P.sor_w;
    D.max_vel = (float)P.max_vel; D.min_depth = (float)P.min_depth; D.dt = (float)P.dt;
    seeds[w] = P.seed;
    // joints: setters in FP64, stored FP32
    std::vector<std::vector<int>> per_body(D.nb);
    for (int j = 0; j < D.njp; ++j) {
      const int gj = D.joint_off + j;
      const int type = sc->joint_type[gj];
      if (type != ODEGPU_JOINT_BALL && type != ODEGPU_JOINT_HINGE && type != ODEGPU_JOINT_HINGE2 &&
          type != ODEGPU_JOINT_SLIDER && type != ODEGPU_JOINT_UNIVERSAL && type != ODEGPU_JOINT_FIXED &&
          type != ODEGPU_JOINT_AMOTOR) {
        delete B;
        return fail(ODEGPU_E_ARG, "unsupported joint type " + std::to_string(type));
      }
      og_host::HJoint H;
      og_host::setup_joint(type, H, hb.data() + D.body_off, sc->joint_body[2 * gj], sc->joint_body[2 * gj + 1],
                           sc->joint_anchor + 3 * (size_t)gj, sc->joint_axis1 + 3 * (size_t)gj,
                           sc->joint_axis2 + 3 * (size_t)gj, sc->joint_param + ODEGPU_JOINT_NPARAM * (size_t)gj);
      DevJoint& J = joints[gj];
      std::memset(&J, 0, sizeof(J));
      J.type = type; J.b1 = H.b1; J.b2 = H.b2; J.reverse = H.reverse;
      pack_joint_geometry(type, H, J);
      const double* jp = sc->joint_param + ODEGPU_JOINT_NPARAM * (size_t)gj;
      auto limot = [&](DevLimot& L, const double* p) {
        // dxJointLimitMotor::init then ::set in parameter order (joint.cpp:456-508)
        L.lostop = (float)p[0]; L.histop = (float)p[1]; L.vel = (float)p[2];
        L.fmax = p[3] >= 0 ? (float)p[3] : 0.f;
        L.fudge = (p[4] >= 0 && p[4] <= 1) ? (float)p[4] : 1.f;
        L.bounce = (float)p[5]; L.normal_cfm = (float)p[6]; L.stop_erp = (float)p[7];
        L.stop_cfm = (float)p[8];
      };
      if (type == ODEGPU_JOINT_BALL || type == ODEGPU_JOINT_FIXED) { J.erp = (float)jp[0]; J.cfm = (float)jp[1]; }
      if (type == ODEGPU_JOINT_HINGE || type == ODEGPU_JOINT_SLIDER) limot(J.lm1, jp);
      if (type == ODEGPU_JOINT_UNIVERSAL) {
        limot(J.lm1, jp);
        limot(J.lm2, jp + 9);
      }
      if (type == ODEGPU_JOINT_AMOTOR) {
        limot(J.lm1, jp + 5);
        limot(J.lm2, jp + 14);
        limot(J.lm3, jp + 23);
      }
      if (type == ODEGPU_JOINT_HINGE2) {
        limot(J.lm1, jp);
        limot(J.lm2, jp + 9);
        J.susp_erp = (float)jp[18];
        J.susp_cfm = (float)jp[19];
      }
      if (J.b1 >= 0) per_body[J.b1].push_back(j);
      if (J.b2 >= 0) per_body[J.b2].push_back(j);
    }
    // persistent adjacency, newest attach first (dJointAttach prepends)
    int* ps = padj_start.data() + D.body_off + w;
    for (int b = 0; b < D.nb; ++b) {
      ps[b] = (int)padj.size();
      for (auto it = per_body[b].rbegin(); it != per_body[b].rend(); ++it) padj.push_back(*it);
    }
    ps[D.nb] = (int)padj.size();
  }
  B->contact_cap_total = contact_off;
  B->row_cap_total = row_off;
  const long long jl_total = (long long)B->nj_total + contact_off;

  int rc = 0;
  rc = rc ? rc : B->world.upload(wd);
  rc = rc ? rc : B->seed.upload(seeds);
  rc = rc ? rc : B->status.upload(std::vector<int>(W, 0));
  rc = rc ? rc : B->ncontacts.upload(std::vector<int>(W, 0));
  rc = rc ? rc : B->nrows.upload(std::vector<int>(W, 0));
  rc = rc ? rc : B->nislands.upload(std::vector<int>(W, 0));
  rc = rc ? rc : B->pos.upload(pos);
  rc = rc ? rc : B->q.upload(q);
  rc = rc ? rc : B->lvel.upload(lv);
  rc = rc ? rc : B->avel.upload(av);
  rc = rc ? rc : B->facc.alloc(NB);
  rc = rc ? rc : B->tacc.alloc(NB);
  rc = rc ? rc : B->mass.upload(mass);
  rc = rc ? rc : B->invMass.upload(invMass);
  rc = rc ? rc : B->I.upload(I);
  rc = rc ? rc : B->invI.upload(invI);
  rc = rc ? rc : B->invIw.alloc(12 * (size_t)NB);
  rc = rc ? rc : B->bflags.upload(flags);
  rc = rc ? rc : B->gtype.upload(gtype);
  rc = rc ? rc : B->gbody.upload(gbody);
  rc = rc ? rc : B->gsurf.upload(gsurf);
  rc = rc ? rc : B->gparam.upload(gparam);
  rc = rc ? rc : B->gpos.upload(gpos);
  rc = rc ? rc : B->hfs.upload(hfs);
  rc = rc ? rc : B->hf_heights.upload(hf_heights);
  rc = rc ? rc : B->gbound.upload(gbound);
  rc = rc ? rc : B->surfaces.upload(surf);
  rc = rc ? rc : B->joints.upload(joints);
  rc = rc ? rc : B->padj_start.upload(padj_start);
  if (padj.empty()) padj.push_back(0);
  rc = rc ? rc : B->padj.upload(padj);
  rc = rc ? rc : B->contacts.alloc(contact_off);
  rc = rc ? rc : B->rows.alloc((size_t)row_off * kRowWords);
  rc = rc ? rc : B->sweep.alloc(((size_t)row_off + 32 * (size_t)W) * 8);
  rc = rc ? rc : B->fwd_scratch.alloc((size_t)std::max(1, n_fwd_scratch) * kFwdScratchPerWorld);
  if (hf_ws_total > 0) rc = rc ? rc : B->hf_ws.alloc((size_t)hf_ws_total);
  rc = rc ? rc : B->jlist.alloc(jl_total);
  rc = rc ? rc : B->jrow.alloc(jl_total);
  rc = rc ? rc : B->jm.alloc(jl_total);
  rc = rc ? rc : B->adj.alloc(2 * jl_total);
  rc = rc ? rc : B->adj_start.alloc((size_t)NB + W);
  rc = rc ? rc : B->island_jstart.alloc((size_t)NB + W);
  rc = rc ? rc : B->island_rstart.alloc((size_t)NB + W);
  rc = rc ? rc : B->state_scratch.alloc((size_t)NB * ODEGPU_BODY_REC);
  if (!rc) rc = set_controls(B, sc->n_ctrl_steps, sc->joint_torque, sc->body_force);
  if (!rc) rc = set_joint_stops(B, sc->n_ctrl_steps, sc->joint_stop);
  if (!rc && cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(ODEGPU_E_CUDA, "stream creation failed");
  if (!rc) {
    // launch order: worlds by decreasing body count (ties by index)
    std::vector<int> ord(W);
    for (int w = 0; w < W; ++w) ord[w] = w;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return wd[a].nb > wd[b].nb; });
    rc = B->order.upload(ord);
  }
  if (!rc && configure_kernels() != 0) rc = fail(ODEGPU_E_CUDA, "cannot configure shared memory");
  for (int k = 0; k < 3; ++k) B->kwpb[k] = std::min(B->warps_per_block, kMaxWpb[k]);
  B->kwpb[4] = std::min(B->warps_per_block, kMaxWpb[4]);
  if (!rc && B->lw) rc = lw_setup(B, sc);
  if (rc) { delete B; return rc; }
  *out = B;
  return 0;
}

void odegpuBatchDestroy(odegpuBatchID b) {
  if (!b) return;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

int odegpuBatchSetControls(odegpuBatchID b, int n_ctrl_steps, const double* jt, const double* bf) {
  if (!b) return fail(ODEGPU_E_ARG, "null batch");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  return set_controls(b, n_ctrl_steps, jt, bf);
}

int odegpuBatchSetJointStops(odegpuBatchID b, int n_ctrl_steps, const double* stops) {
  if (!b || n_ctrl_steps < 0) return fail(ODEGPU_E_ARG, "bad arguments");
  if (b->n_ctrl_steps > 0 && n_ctrl_steps != b->n_ctrl_steps && (b->joint_torque.p || b->body_force.p))
    return fail(ODEGPU_E_ARG, "joint stops must cover the same number of control steps as the torques/forces");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  if (n_ctrl_steps > 0) b->n_ctrl_steps = n_ctrl_steps;
  return set_joint_stops(b, n_ctrl_steps, stops);
}

int odegpuBatchSetStepIndex(odegpuBatchID b, int step) {
  if (!b || step < 0) return fail(ODEGPU_E_ARG, "bad arguments");
  b->step_counter = step;
  return 0;
}

int odegpuBatchStep(odegpuBatchID b, int n_steps) {
  if (!b || n_steps < 0) return fail(ODEGPU_E_ARG, "bad arguments");
  if (n_steps == 0) return 0;
  OG_CUDA(cudaSetDevice(b->device));
  StepOptions opt{1, nullptr, nullptr, nullptr, 0, 0};
  if (int rc = b->launch(0, b->n_worlds, n_steps, opt)) return rc;
  b->step_counter += n_steps;
  return 0;
}

int odegpuBatchStepPlain(odegpuBatchID b, int n_steps) {
  if (!b || n_steps < 0) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  StepOptions opt{1, nullptr, nullptr, nullptr, 0, 0};
  b->single_world = true;
  for (int w = 0; w < b->n_worlds; ++w) {
    for (int s = 0; s < n_steps; ++s) {
      const int base = b->step_counter;
      b->step_counter = base + s;
      const int rc = b->launch(w, 1, 1, opt, false);
      b->step_counter = base;
      if (rc) { b->single_world = false; return rc; }
    }
  }
  b->single_world = false;
  b->step_counter += n_steps;
  return 0;
}

int odegpuBatchStepGraph(odegpuBatchID b, int n_steps) {
  if (!b || n_steps < 0) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  StepOptions opt{1, nullptr, nullptr, nullptr, 0, 0};
  if (b->exact)
    if (int rc = b->ensure_exact_by_capacity()) return rc;
  cudaGraph_t graph;
  OG_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  for (int s = 0; s < n_steps; ++s) {
    const int base = b->step_counter;
    b->step_counter = base + s;
    const int rc = b->launch(0, b->n_worlds, 1, opt);
    b->step_counter = base;
    if (rc) { cudaStreamEndCapture(b->stream, &graph); return rc; }
  }
  OG_CUDA(cudaStreamEndCapture(b->stream, &graph));
  cudaGraphExec_t exec;
  OG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  const cudaError_t e = cudaGraphLaunch(exec, b->stream);
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(ODEGPU_E_CUDA, cudaGetErrorString(e));
  b->step_counter += n_steps;
  return 0;
}

int odegpuBatchSetStepper(odegpuBatchID b, int exact) {
  if (!b || (exact != 0 && exact != 1)) return fail(ODEGPU_E_ARG, "bad arguments");
  if (exact && b->lw) return fail(ODEGPU_E_ARG, "dWorldStep is not available for a large world");
  b->exact = exact != 0;
  return 0;
}

int odegpuBatchSetTiming(odegpuBatchID b, int on) {
  if (!b) return fail(ODEGPU_E_ARG, "null batch");
  b->timing = on != 0;
  b->ev_used = 0;
  return 0;
}

int odegpuBatchGetKernelTimes(odegpuBatchID b, double* ms, long long* n_steps) {
  if (!b || !ms) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  ms[0] = ms[1] = ms[2] = 0.0;
  const size_t steps = b->ev_used / 4;
  for (size_t k = 0; k < steps; ++k) {
    for (int j = 0; j < 3; ++j) {
      float t = 0.f;
      OG_CUDA(cudaEventElapsedTime(&t, b->ev_pool[4 * k + j], b->ev_pool[4 * k + j + 1]));
      ms[j] += t;
    }
  }
  if (n_steps) *n_steps = (long long)steps;
  b->ev_used = 0;
  return 0;
}

int odegpuBatchSetFeedback(odegpuBatchID b, int on) {
  if (!b) return fail(ODEGPU_E_ARG, "null batch");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  if (on && !b->feedback.p) {
    if (int rc = b->jcopy.alloc((size_t)std::max<long long>(1, b->row_cap_total) * 12)) return rc;
    if (int rc = b->feedback.alloc((size_t)std::max(1, b->nj_total) * 12)) return rc;
    OG_CUDA(cudaMemset(b->feedback.p, 0, (size_t)std::max(1, b->nj_total) * 12 * sizeof(float)));
  }
  b->feedback_on = on != 0;
  return 0;
}

int odegpuBatchGetFeedback(odegpuBatchID b, double* out) {
  if (!b || !out) return fail(ODEGPU_E_ARG, "bad arguments");
  if (!b->feedback.p) return fail(ODEGPU_E_ARG, "feedback is not enabled (odegpuBatchSetFeedback)");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  std::vector<float> tmp((size_t)b->nj_total * 12);
  if (!tmp.empty())
    OG_CUDA(cudaMemcpy(tmp.data(), b->feedback.p, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < tmp.size(); ++i) out[i] = tmp[i];
  return 0;
}

int odegpuBatchSetLaunchConfig(odegpuBatchID b, int kernel, int warps_per_block, int smem_carveout) {
  if (!b || kernel < 0 || kernel > 4) return fail(ODEGPU_E_ARG, "bad kernel index");
  if (warps_per_block < 1 || warps_per_block > kMaxWpb[kernel])
    return fail(ODEGPU_E_ARG, "warps per block out of range for this kernel");
  if (smem_carveout < -1 || smem_carveout > 100) return fail(ODEGPU_E_ARG, "carveout must be -1 or 0..100");
  b->kwpb[kernel] = warps_per_block;
  b->kcarve[kernel] = smem_carveout;
  return 0;
}

int odegpuBatchSetLaunchConfigEx(odegpuBatchID b, int kernel, int warps_per_block, int smem_carveout,
                                 int variant) {
  if (!b || (variant != 0 && !(kernel == 2 && variant == 1)))
    return fail(ODEGPU_E_ARG, "variant 1 exists for the solve kernel (2) only");
  if (int rc = odegpuBatchSetLaunchConfig(b, kernel, warps_per_block, smem_carveout)) return rc;
  if (kernel == 2) b->solve_lowreg = variant == 1;
  return 0;
}

int odegpuBatchGetLaunchConfigEx(odegpuBatchID b, int kernel, int* warps_per_block, int* smem_carveout,
                                 int* variant) {
  if (!b || kernel < 0 || kernel > 4) return fail(ODEGPU_E_ARG, "bad kernel index");
  if (warps_per_block) *warps_per_block = b->kwpb[kernel];
  if (smem_carveout) *smem_carveout = b->kcarve[kernel];
  if (variant) *variant = (kernel == 2 && b->solve_lowreg) ? 1 : 0;
  return 0;
}

int odegpuBatchSetStepKernels(odegpuBatchID b, int fused) {
  if (!b || (fused != 0 && fused != 1)) return fail(ODEGPU_E_ARG, "bad arguments");
  b->fused = fused != 0;
  return 0;
}

int odegpuBatchGetStepKernels(odegpuBatchID b, int* fused, int* warps_per_block, int* smem_carveout) {
  if (!b || !fused) return fail(ODEGPU_E_ARG, "bad arguments");
  *fused = b->fused ? 1 : 0;
  if (warps_per_block) *warps_per_block = b->kwpb[4];
  if (smem_carveout) *smem_carveout = b->kcarve[4];
  return 0;
}

int odegpuBatchAutotune(odegpuBatchID b, int n_steps) {
  if (b && b->lw) return fail(ODEGPU_E_ARG, "not available for a large world (one world above the on-chip limits)");
  if (b && b->exact) return fail(ODEGPU_E_ARG, "not available with the dWorldStep stepper (odegpuBatchSetStepper)");
  if (!b || n_steps < 1) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  const size_t rec = (size_t)b->nb_total * ODEGPU_BODY_REC;
  DBuf<float> st;
  DBuf<unsigned> sd;
  if (int rc = st.alloc(rec)) return rc;
  if (int rc = sd.alloc((size_t)b->n_worlds)) return rc;
  b->pack_to(st.p);
  OG_CUDA(cudaMemcpyAsync(sd.p, b->seed.p, b->n_worlds * sizeof(unsigned), cudaMemcpyDeviceToDevice, b->stream));
  const int saved_counter = b->step_counter;
  const bool saved_timing = b->timing;
  auto restore = [&]() -> int {
    b->unpack_from(st.p);
    OG_CUDA(cudaMemcpyAsync(b->seed.p, sd.p, b->n_worlds * sizeof(unsigned), cudaMemcpyDeviceToDevice,
                            b->stream));
    b->step_counter = saved_counter;
    return 0;
  };
  static const int kWpb[] = {1, 2, 4, 8};
  static const int kCarve[] = {-1, 25, 50, 75, 100};
  double best[3] = {INFINITY, INFINITY, INFINITY};
  int best_w[3] = {b->kwpb[0], b->kwpb[1], b->kwpb[2]}, best_c[3] = {b->kcarve[0], b->kcarve[1], b->kcarve[2]};
  StepOptions opt{1, nullptr, nullptr, nullptr, 0, 0};
  b->timing = true;
  const bool saved_fused = b->fused, saved_lowreg = b->solve_lowreg;
  b->fused = false;
  bool best_lowreg = saved_lowreg;
  int rc = 0;
  // every shape of the three kernels with the 168-register solve kernel, then
  // the solve kernel's shapes with its 128-register budget
  for (int v = 0; v < 2 && !rc; ++v)
  for (int wi = 0; wi < 4 && !rc; ++wi) {
    for (int ci = 0; ci < 5 && !rc; ++ci) {
      bool tried[3];
      b->solve_lowreg = v == 1;
      for (int k = 0; k < 3; ++k) {
        tried[k] = kWpb[wi] <= kMaxWpb[k] && (v == 0 || k == 2);
        b->kwpb[k] = tried[k] ? kWpb[wi] : best_w[k];
        b->kcarve[k] = tried[k] ? kCarve[ci] : best_c[k];
      }
      if ((rc = restore())) break;
      if ((rc = b->launch(0, b->n_worlds, 1, opt))) break;       // warm-up step (not counted)
      b->ev_used = 0;
      if ((rc = b->launch(0, b->n_worlds, n_steps, opt))) break;
      if (cudaStreamSynchronize(b->stream) != cudaSuccess) { rc = fail(ODEGPU_E_CUDA, "autotune step"); break; }
      double ms[3] = {0, 0, 0};
      for (size_t q = 0; q + 3 < b->ev_used; q += 4)
        for (int k = 0; k < 3; ++k) {
          float t = 0.f;
          cudaEventElapsedTime(&t, b->ev_pool[q + k], b->ev_pool[q + k + 1]);
          ms[k] += t;
        }
      for (int k = 0; k < 3; ++k)
        if (tried[k] && ms[k] < best[k]) {
          best[k] = ms[k];
          best_w[k] = kWpb[wi];
          best_c[k] = kCarve[ci];
          if (k == 2) best_lowreg = v == 1;
        }
    }
  }
  for (int k = 0; k < 3; ++k) { b->kwpb[k] = best_w[k]; b->kcarve[k] = best_c[k]; }
  b->solve_lowreg = rc ? saved_lowreg : best_lowreg;
  // the fused step kernel: its shapes against the best split step (the sum of
  // the three kernels' best times)
  double best_f = INFINITY;
  int best_fw = b->kwpb[4], best_fc = b->kcarve[4];
  b->fused = true;
  for (int wi = 0; wi < 4 && !rc; ++wi) {
    if (kWpb[wi] > kMaxWpb[4]) continue;
    for (int ci = 0; ci < 5 && !rc; ++ci) {
      b->kwpb[4] = kWpb[wi];
      b->kcarve[4] = kCarve[ci];
      if ((rc = restore())) break;
      if ((rc = b->launch(0, b->n_worlds, 1, opt))) break;
      b->ev_used = 0;
      if ((rc = b->launch(0, b->n_worlds, n_steps, opt))) break;
      if (cudaStreamSynchronize(b->stream) != cudaSuccess) { rc = fail(ODEGPU_E_CUDA, "autotune step"); break; }
      double ms = 0.0;
      for (size_t q = 0; q + 3 < b->ev_used; q += 4) {
        float t = 0.f;
        cudaEventElapsedTime(&t, b->ev_pool[q], b->ev_pool[q + 1]);
        ms += t;
      }
      if (ms < best_f) { best_f = ms; best_fw = kWpb[wi]; best_fc = kCarve[ci]; }
    }
  }
  b->kwpb[4] = best_fw;
  b->kcarve[4] = best_fc;
  b->fused = rc ? saved_fused : best_f < best[0] + best[1] + best[2];
  b->ev_used = 0;
  b->timing = saved_timing;
  if (!rc) rc = restore();
  if (!rc && cudaStreamSynchronize(b->stream) != cudaSuccess) rc = fail(ODEGPU_E_CUDA, "autotune restore");
  return rc;
}

int odegpuBatchGetLaunchConfig(odegpuBatchID b, int* cfg) {
  if (!b || !cfg) return fail(ODEGPU_E_ARG, "bad arguments");
  for (int k = 0; k < 4; ++k) { cfg[2 * k] = b->kwpb[k]; cfg[2 * k + 1] = b->kcarve[k]; }
  return 0;
}

int odegpuBatchGetLaunchCount(odegpuBatchID b, long long* launches) {
  if (!b || !launches) return fail(ODEGPU_E_ARG, "bad arguments");
  *launches = b->launches;
  return 0;
}

int odegpuBatchSetControlsF32(odegpuBatchID b, int n_ctrl_steps, const float* jt, const float* bf) {
  if (!b || n_ctrl_steps < 0) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  if (b->joint_torque.p) { cudaFree(b->joint_torque.p); b->joint_torque.p = nullptr; }
  if (b->body_force.p) { cudaFree(b->body_force.p); b->body_force.p = nullptr; }
  b->n_ctrl_steps = n_ctrl_steps;
  if (n_ctrl_steps == 0) return 0;
  const size_t nt = (size_t)n_ctrl_steps * b->nj_total * 2, nf = (size_t)n_ctrl_steps * b->nb_total * 6;
  if (jt) {
    if (int rc = b->joint_torque.alloc(nt)) return rc;
    OG_CUDA(cudaMemcpy(b->joint_torque.p, jt, nt * sizeof(float), cudaMemcpyDefault));
  }
  if (bf) {
    if (int rc = b->body_force.alloc(nf)) return rc;
    OG_CUDA(cudaMemcpy(b->body_force.p, bf, nf * sizeof(float), cudaMemcpyDefault));
  }
  return 0;
}

int odegpuBatchRolloutForward(odegpuBatchID b, int n_steps, int ckpt_every) {
  if (b && b->lw) return fail(ODEGPU_E_ARG, "not available for a large world (one world above the on-chip limits)");
  if (b && b->exact) return fail(ODEGPU_E_ARG, "not available with the dWorldStep stepper (odegpuBatchSetStepper)");
  if (!b || n_steps <= 0 || ckpt_every <= 0) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  auto& R = b->ro;
  const size_t rec = (size_t)b->nb_total * ODEGPU_BODY_REC;
  const int n_ckpt = (n_steps + ckpt_every - 1) / ckpt_every;
  R.valid = 0;
  if (R.ckpt_state.n < (size_t)n_ckpt * rec) {
    if (R.ckpt_state.p) { cudaFree(R.ckpt_state.p); R.ckpt_state.p = nullptr; }
    if (int rc = R.ckpt_state.alloc((size_t)n_ckpt * rec)) return rc;
  }
  if (R.ckpt_seed.n < (size_t)n_ckpt * b->n_worlds) {
    if (R.ckpt_seed.p) { cudaFree(R.ckpt_seed.p); R.ckpt_seed.p = nullptr; }
    if (int rc = R.ckpt_seed.alloc((size_t)n_ckpt * b->n_worlds)) return rc;
  }
  if (!R.final_state.p && R.final_state.alloc(rec)) return ODEGPU_E_NOMEM;
  if (!R.final_seed.p && R.final_seed.alloc(b->n_worlds)) return ODEGPU_E_NOMEM;
  R.n_steps = n_steps;
  R.ckpt = ckpt_every;
  R.start = b->step_counter;
  StepOptions opt{1, nullptr, nullptr, nullptr, 0, 0};
  for (int s = 0; s < n_steps; ++s) {
    if (s % ckpt_every == 0) {
      const int c = s / ckpt_every;
      b->pack_to(R.ckpt_state.p + (size_t)c * rec);
      OG_CUDA(cudaMemcpyAsync(R.ckpt_seed.p + (size_t)c * b->n_worlds, b->seed.p, b->n_worlds * sizeof(unsigned),
                              cudaMemcpyDeviceToDevice, b->stream));
    }
    if (int rc = b->launch(0, b->n_worlds, 1, opt)) return rc;
    b->step_counter += 1;
  }
  b->pack_to(R.final_state.p);
  OG_CUDA(cudaMemcpyAsync(R.final_seed.p, b->seed.p, b->n_worlds * sizeof(unsigned), cudaMemcpyDeviceToDevice,
                          b->stream));
  OG_CUDA(cudaGetLastError());
  R.valid = 1;
  return 0;
}

int odegpuBatchRolloutBackward(odegpuBatchID b, const float* grad_final, float* grad_init, float* grad_jt,
                               float* grad_bf) {
  if (b && b->lw) return fail(ODEGPU_E_ARG, "not available for a large world (one world above the on-chip limits)");
  if (b && b->exact) return fail(ODEGPU_E_ARG, "not available with the dWorldStep stepper (odegpuBatchSetStepper)");
  if (!b || !grad_final) return fail(ODEGPU_E_ARG, "bad arguments");
  auto& R = b->ro;
  if (!R.valid) return fail(ODEGPU_E_ARG, "no rollout recorded (odegpuBatchRolloutForward)");
  OG_CUDA(cudaSetDevice(b->device));
  const size_t rec = (size_t)b->nb_total * ODEGPU_BODY_REC;
  int iters_max = 1;
  for (const WorldDesc& D : b->h_world) iters_max = std::max(iters_max, D.iterations);
  const int rounds_max = (iters_max + 7) / 8;
  const size_t rcap = (size_t)std::max<long long>(1, b->row_cap_total);
  auto need = [](auto& buf, size_t n) -> int {
    if (buf.n >= n && buf.p) return 0;
    if (buf.p) { cudaFree(buf.p); buf.p = nullptr; }
    return buf.alloc(n);
  };
  if (need(R.seg_state, (size_t)R.ckpt * rec) || need(R.seg_seed, (size_t)R.ckpt * b->n_worlds) ||
      need(R.state_bar, rec) || need(R.body_tmp, (size_t)b->nb_total * kAdjBody) ||
      need(R.row_tmp, rcap * kAdjRow) || need(R.lam_tape, rcap * iters_max) ||
      need(R.code_tape, rcap * iters_max) || need(R.seq_tape, rcap * rounds_max) ||
      need(R.dbg, rcap * kRowWords) || need(R.status, (size_t)b->n_worlds))
    return ODEGPU_E_NOMEM;
  OG_CUDA(cudaMemsetAsync(R.status.p, 0, b->n_worlds * sizeof(int), b->stream));
  OG_CUDA(cudaMemcpyAsync(R.state_bar.p, grad_final, rec * sizeof(float), cudaMemcpyDefault, b->stream));
  const int nctrl = b->n_ctrl_steps;
  if (grad_jt && nctrl > 0)
    OG_CUDA(cudaMemsetAsync(grad_jt, 0, (size_t)nctrl * b->nj_total * 2 * sizeof(float), b->stream));
  if (grad_bf && nctrl > 0)
    OG_CUDA(cudaMemsetAsync(grad_bf, 0, (size_t)nctrl * b->nb_total * 6 * sizeof(float), b->stream));
  AdjDev a;
  a.state_bar = R.state_bar.p; a.body_tmp = R.body_tmp.p; a.row_tmp = R.row_tmp.p;
  a.lam_tape = R.lam_tape.p; a.code_tape = R.code_tape.p; a.seq_tape = R.seq_tape.p; a.dbg = R.dbg.p;
  a.g_jt = nctrl > 0 ? grad_jt : nullptr;
  a.g_bf = nctrl > 0 ? grad_bf : nullptr;
  a.status = R.status.p;
  a.iters_max = iters_max;
  a.rounds_max = rounds_max;
  StepOptions fwd{1, nullptr, nullptr, nullptr, 0, 0};
  StepOptions tap{1, R.dbg.p, nullptr, nullptr, 0, 0};
  const int saved_counter = b->step_counter;
  const int n_ckpt = (R.n_steps + R.ckpt - 1) / R.ckpt;
  for (int c = n_ckpt - 1; c >= 0; --c) {
    const int s0 = c * R.ckpt, len = std::min(R.ckpt, R.n_steps - s0);
    // recompute the segment from its checkpoint, keeping every pre-step state
    b->unpack_from(R.ckpt_state.p + (size_t)c * rec);
    OG_CUDA(cudaMemcpyAsync(b->seed.p, R.ckpt_seed.p + (size_t)c * b->n_worlds, b->n_worlds * sizeof(unsigned),
                            cudaMemcpyDeviceToDevice, b->stream));
    for (int j = 0; j < len; ++j) {
      b->pack_to(R.seg_state.p + (size_t)j * rec);
      OG_CUDA(cudaMemcpyAsync(R.seg_seed.p + (size_t)j * b->n_worlds, b->seed.p, b->n_worlds * sizeof(unsigned),
                              cudaMemcpyDeviceToDevice, b->stream));
      if (j + 1 < len) {
        b->step_counter = R.start + s0 + j;
        if (int rc = b->launch(0, b->n_worlds, 1, fwd)) { b->step_counter = saved_counter; return rc; }
      }
    }
    // the segment's steps backwards
    for (int j = len - 1; j >= 0; --j) {
      const int step = R.start + s0 + j;
      b->unpack_from(R.seg_state.p + (size_t)j * rec);
      OG_CUDA(cudaMemcpyAsync(b->seed.p, R.seg_seed.p + (size_t)j * b->n_worlds, b->n_worlds * sizeof(unsigned),
                              cudaMemcpyDeviceToDevice, b->stream));
      if (int rc = b->launch_setup(step, tap)) { b->step_counter = saved_counter; return rc; }
      b->apply_carveout(3);
      adjoint_step_kernel<<<b->nblocks(b->n_worlds, 3), b->kwpb[3] * 32, b->kwpb[3] * (size_t)kAdjSmemPerWarp,
                            b->stream>>>(b->dev(), a, step);
      b->launches += 1;
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) {
        b->step_counter = saved_counter;
        return fail(ODEGPU_E_CUDA, std::string("adjoint launch: ") + cudaGetErrorString(e));
      }
    }
  }
  if (grad_init)
    OG_CUDA(cudaMemcpyAsync(grad_init, R.state_bar.p, rec * sizeof(float), cudaMemcpyDefault, b->stream));
  // leave the batch where the forward rollout ended
  b->unpack_from(R.final_state.p);
  OG_CUDA(cudaMemcpyAsync(b->seed.p, R.final_seed.p, b->n_worlds * sizeof(unsigned), cudaMemcpyDeviceToDevice,
                          b->stream));
  b->step_counter = saved_counter;
  OG_CUDA(cudaGetLastError());
  return 0;
}

int odegpuBatchAdjointStatus(odegpuBatchID b, int* status) {
  if (!b || !status) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  if (!b->ro.status.p) { std::memset(status, 0, b->n_worlds * sizeof(int)); return 0; }
  OG_CUDA(cudaMemcpy(status, b->ro.status.p, b->n_worlds * sizeof(int), cudaMemcpyDeviceToHost));
  return 0;
}

int odegpuBatchSynchronize(odegpuBatchID b) {
  if (!b) return fail(ODEGPU_E_ARG, "null batch");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  return 0;
}

int odegpuBatchReadStateF32Async(odegpuBatchID b, float* state) {
  if (!b || !state) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  const int nb = b->nb_total;
  pack_state_kernel<<<(nb + 255) / 256, 256, 0, b->stream>>>(b->dev(), nb, b->state_scratch.p);
  b->launches += 1;
  OG_CUDA(cudaGetLastError());
  OG_CUDA(cudaMemcpyAsync(state, b->state_scratch.p, (size_t)nb * ODEGPU_BODY_REC * sizeof(float),
                          cudaMemcpyDefault, b->stream));
  return 0;
}

int odegpuBatchWriteStateF32Async(odegpuBatchID b, const float* state) {
  if (!b || !state) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  const int nb = b->nb_total;
  OG_CUDA(cudaMemcpyAsync(b->state_scratch.p, state, (size_t)nb * ODEGPU_BODY_REC * sizeof(float),
                          cudaMemcpyDefault, b->stream));
  unpack_state_kernel<<<(nb + 255) / 256, 256, 0, b->stream>>>(b->dev(), nb, b->state_scratch.p);
  b->launches += 1;
  OG_CUDA(cudaGetLastError());
  return 0;
}

int odegpuBatchReadState(odegpuBatchID b, double* state) {
  if (!b || !state) return fail(ODEGPU_E_ARG, "bad arguments");
  std::vector<float> tmp((size_t)b->nb_total * ODEGPU_BODY_REC);
  if (int rc = odegpuBatchReadStateF32Async(b, tmp.data())) return rc;
  OG_CUDA(cudaStreamSynchronize(b->stream));
  for (size_t i = 0; i < tmp.size(); ++i) state[i] = tmp[i];
  return 0;
}

int odegpuBatchWriteState(odegpuBatchID b, const double* state) {
  if (!b || !state) return fail(ODEGPU_E_ARG, "bad arguments");
  std::vector<float> tmp((size_t)b->nb_total * ODEGPU_BODY_REC);
  for (size_t i = 0; i < tmp.size(); ++i) tmp[i] = (float)state[i];
  // quaternions are normalised on the way in, as dBodySetQuaternion does
  for (int k = 0; k < b->nb_total; ++k) {
    double qd[4];
    for (int j = 0; j < 4; ++j) qd[j] = state[(size_t)k * ODEGPU_BODY_REC + 3 + j];
    og_host::normalize4(qd);
    for (int j = 0; j < 4; ++j) tmp[(size_t)k * ODEGPU_BODY_REC + 3 + j] = (float)qd[j];
  }
  if (int rc = odegpuBatchWriteStateF32Async(b, tmp.data())) return rc;
  OG_CUDA(cudaStreamSynchronize(b->stream));
  return 0;
}

static int copy_ints(odegpuBatchID b, const int* src, int* dst, size_t n) {
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  return 0;
}

int odegpuBatchGetStatus(odegpuBatchID b, int* status) {
  if (!b || !status) return fail(ODEGPU_E_ARG, "bad arguments");
  return copy_ints(b, b->status.p, status, b->n_worlds);
}

int odegpuBatchGetCounts(odegpuBatchID b, int* nc, int* nr, int* ni) {
  if (!b) return fail(ODEGPU_E_ARG, "bad arguments");
  if (nc) if (int rc = copy_ints(b, b->ncontacts.p, nc, b->n_worlds)) return rc;
  if (nr) if (int rc = copy_ints(b, b->nrows.p, nr, b->n_worlds)) return rc;
  if (ni) if (int rc = copy_ints(b, b->nislands.p, ni, b->n_worlds)) return rc;
  return 0;
}

int odegpuBatchGetSeeds(odegpuBatchID b, unsigned int* seeds) {
  if (!b || !seeds) return fail(ODEGPU_E_ARG, "bad arguments");
  return copy_ints(b, reinterpret_cast<const int*>(b->seed.p), reinterpret_cast<int*>(seeds), b->n_worlds);
}

int odegpuBatchSetSeeds(odegpuBatchID b, const unsigned int* seeds) {
  if (!b || !seeds) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaMemcpyAsync(b->seed.p, seeds, b->n_worlds * sizeof(unsigned), cudaMemcpyHostToDevice, b->stream));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  return 0;
}

int odegpuBatchInfo(odegpuBatchID b, int* n_worlds, int* nb_total, int* nj_total, long long* row_cap,
                    long long* contact_cap) {
  if (!b) return fail(ODEGPU_E_ARG, "null batch");
  if (n_worlds) *n_worlds = b->n_worlds;
  if (nb_total) *nb_total = b->nb_total;
  if (nj_total) *nj_total = b->nj_total;
  if (row_cap) *row_cap = b->row_cap_total;
  if (contact_cap) *contact_cap = b->contact_cap_total;
  return 0;
}

void* odegpuBatchStream(odegpuBatchID b) { return b ? (void*)b->stream : nullptr; }

int odegpuBatchRayCastAsync(odegpuBatchID b, const odegpuRay* d_rays, int n, int flags, odegpuRayHit* d_hits) {
  if (!b || n < 0 || (n > 0 && (!d_rays || !d_hits))) return fail(ODEGPU_E_ARG, "bad arguments");
  const int maxc = flags & 0xffff;
  if (maxc < 1 || maxc > 8) return fail(ODEGPU_E_ARG, "ray casts take 1 to 8 contacts per geom");
  if (n == 0) return 0;
  OG_CUDA(cudaSetDevice(b->device));
  constexpr int kThreads = 128;   // 4 rays per block, one warp each
  const long long blocks = ((long long)n * 32 + kThreads - 1) / kThreads;
  raycast_kernel<<<(unsigned)blocks, kThreads, 0, b->stream>>>(b->dev(), d_rays, nullptr, n, (unsigned)flags, d_hits,
                                                                RayBig{nullptr, 0, 0});
  b->launches += 1;
  OG_CUDA(cudaGetLastError());
  return 0;
}

int odegpuBatchRayCast(odegpuBatchID b, const odegpuRay* rays, int n, int flags, odegpuRayHit* hits) {
  if (!b || n < 0 || (n > 0 && (!rays || !hits))) return fail(ODEGPU_E_ARG, "bad arguments");
  for (int i = 0; i < n; ++i) {
    const odegpuRay& r = rays[i];
    if (r.world < 0 || r.world >= b->n_worlds) return fail(ODEGPU_E_ARG, "ray " + std::to_string(i) + ": bad world");
    if (r.body >= b->h_world[r.world].nb) return fail(ODEGPU_E_ARG, "ray " + std::to_string(i) + ": bad body");
    if (!std::isfinite(r.length) || r.length < 0)
      return fail(ODEGPU_E_ARG, "ray " + std::to_string(i) + ": length must be finite and >= 0");
  }
  if (n == 0) return 0;
  OG_CUDA(cudaSetDevice(b->device));
  if (b->ray_in.n < (size_t)n) {
    cudaFree(b->ray_in.p); b->ray_in.p = nullptr;
    cudaFree(b->ray_out.p); b->ray_out.p = nullptr;
    if (int rc = b->ray_in.alloc(n)) return rc;
    if (int rc = b->ray_out.alloc(n)) return rc;
  }
  OG_CUDA(cudaMemcpyAsync(b->ray_in.p, rays, (size_t)n * sizeof(odegpuRay), cudaMemcpyHostToDevice, b->stream));
  if (int rc = odegpuBatchRayCastAsync(b, b->ray_in.p, n, flags, b->ray_out.p)) return rc;
  OG_CUDA(cudaMemcpyAsync(hits, b->ray_out.p, (size_t)n * sizeof(odegpuRayHit), cudaMemcpyDeviceToHost,
                          b->stream));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  // rays whose heightfield zone exceeded the lane's arrays: cast again with
  // a workspace per warp, sized by the longest of them on the finest field
  std::vector<int> again;
  for (int i = 0; i < n; ++i)
    if (hits[i].geom == -3) again.push_back(i);
  if (!again.empty() && b->hf_min_spacing > 0.0) {
    double longest = 0.0;
    for (int i : again) longest = std::max(longest, (double)rays[i].length);
    const int side = std::min(kHFBigZone, hf_zone_side(0.5 * longest, b->hf_min_spacing));
    const int warps = std::min<int>((int)again.size(), 256);
    const long long stride = (hf_ws_bytes(side) + 255) & ~255LL;
    auto grow_buf = [](auto& buf, size_t cnt) -> int {
      if (buf.p && buf.n >= cnt) return 0;
      if (buf.p) { cudaFree(buf.p); buf.p = nullptr; }
      return buf.alloc(cnt);
    };
    if (int rc = grow_buf(b->ray_ws, (size_t)(stride * warps))) return rc;
    if (int rc = grow_buf(b->ray_list, again.size())) return rc;
    OG_CUDA(cudaMemcpyAsync(b->ray_list.p, again.data(), again.size() * sizeof(int), cudaMemcpyHostToDevice,
                            b->stream));
    constexpr int kThreads = 128;
    raycast_kernel<<<(unsigned)((warps * 32 + kThreads - 1) / kThreads), kThreads, 0, b->stream>>>(
        b->dev(), b->ray_in.p, b->ray_list.p, (int)again.size(), (unsigned)flags, b->ray_out.p,
        RayBig{b->ray_ws.p, stride, side});
    b->launches += 1;
    OG_CUDA(cudaGetLastError());
    OG_CUDA(cudaMemcpyAsync(hits, b->ray_out.p, (size_t)n * sizeof(odegpuRayHit), cudaMemcpyDeviceToHost,
                            b->stream));
    OG_CUDA(cudaStreamSynchronize(b->stream));
  }
  int nhit = 0;
  for (int i = 0; i < n; ++i) nhit += hits[i].geom >= 0;
  return nhit;
}

int odegpuBatchLargeWorldStats(odegpuBatchID b, long long* out, int n, int reset) {
  if (!b || !out || n < 0) return fail(ODEGPU_E_ARG, "bad arguments");
  if (!b->lw) return fail(ODEGPU_E_ARG, "the batch has no large world");
  OG_CUDA(cudaSetDevice(b->device));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  unsigned long long v[9];
  OG_CUDA(cudaMemcpy(v, b->lw->stats.p, sizeof(v), cudaMemcpyDeviceToHost));
  for (int k = 0; k < n && k < 9; ++k) out[k] = (long long)v[k];
  if (reset) OG_CUDA(cudaMemset(b->lw->stats.p, 0, sizeof(v)));
  return 0;
}

int odegpuBatchStepTap(odegpuBatchID b, float* rows, float* lambda, float* fc, int* row_off) {
  if (b && b->lw) return fail(ODEGPU_E_ARG, "not available for a large world (one world above the on-chip limits)");
  if (b && b->exact) return fail(ODEGPU_E_ARG, "not available with the dWorldStep stepper (odegpuBatchSetStepper)");
  if (!b) return fail(ODEGPU_E_ARG, "null batch");
  OG_CUDA(cudaSetDevice(b->device));
  DBuf<float> drows, dlam, dfc;
  if (int rc = drows.alloc((size_t)b->row_cap_total * kRowWords)) return rc;
  if (int rc = dlam.alloc(b->row_cap_total)) return rc;
  if (int rc = dfc.alloc((size_t)b->nb_total * 6)) return rc;
  OG_CUDA(cudaMemsetAsync(dfc.p, 0, (size_t)b->nb_total * 6 * sizeof(float), b->stream));
  StepOptions opt{1, drows.p, dlam.p, dfc.p, 0, 0};
  if (int rc = b->launch(0, b->n_worlds, 1, opt)) return rc;
  b->step_counter += 1;
  if (rows)
    OG_CUDA(cudaMemcpyAsync(rows, drows.p, (size_t)b->row_cap_total * kRowWords * sizeof(float),
                            cudaMemcpyDeviceToHost, b->stream));
  if (lambda)
    OG_CUDA(cudaMemcpyAsync(lambda, dlam.p, (size_t)b->row_cap_total * sizeof(float),
                            cudaMemcpyDeviceToHost, b->stream));
  if (fc)
    OG_CUDA(cudaMemcpyAsync(fc, dfc.p, (size_t)b->nb_total * 6 * sizeof(float), cudaMemcpyDeviceToHost,
                            b->stream));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  if (row_off)
    for (int w = 0; w < b->n_worlds; ++w) row_off[w] = b->h_world[w].row_off;
  return 0;
}

int odegpuBatchGetContacts(odegpuBatchID b, int w, float* out, int cap) {
  if (!b || w < 0 || w >= b->n_worlds || (!out && cap > 0)) return fail(ODEGPU_E_ARG, "bad arguments");
  OG_CUDA(cudaSetDevice(b->device));
  int nc = 0;
  OG_CUDA(cudaMemcpyAsync(&nc, b->ncontacts.p + w, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  OG_CUDA(cudaStreamSynchronize(b->stream));
  const int n = std::min(nc, cap);
  if (n > 0) {
    std::vector<DevContact> tmp(n);
    OG_CUDA(cudaMemcpy(tmp.data(), b->contacts.p + b->h_world[w].contact_off, n * sizeof(DevContact),
                       cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) {
      float* o = out + 9 * i;
      const DevContact& c = tmp[i];
      o[0] = c.pos[0]; o[1] = c.pos[1]; o[2] = c.pos[2];
      // report the normal as dCollide returned it (before the attach swap)
      o[3] = c.normal[0]; o[4] = c.normal[1]; o[5] = c.normal[2];
      o[6] = c.depth;
      o[7] = (float)(c.reverse ? -1 : c.b1);
      o[8] = (float)(c.reverse ? c.b1 : c.b2);
    }
  }
  return nc;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Single-world context for the ODE-compatible API (ode_api.cpp).

#include "engine_internal.hpp"

namespace {

__global__ void collide_pair_kernel(GeomView a, GeomView b, unsigned flags, Contact* out, int* n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    Contact c[8];
    const int k = collide_primitive(a, b, flags, c);
    for (int i = 0; i < k; ++i) out[i] = c[i];
    *n = k;
  }
}

template <class T>
int grow(DBuf<T>& b, size_t n) {
  if (b.p && b.n >= n) return 0;
  if (b.p) { cudaFree(b.p); b.p = nullptr; }
  return b.alloc(std::max<size_t>(n, 16));
}
template <class T>
int put(DBuf<T>& b, const std::vector<T>& v, cudaStream_t s, size_t min_cap = 0) {
  if (int rc = grow(b, std::max(v.size(), min_cap))) return rc;
  if (!v.empty() && cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return fail(ODEGPU_E_CUDA, "upload failed");
  return 0;
}

}  // namespace

namespace og {

struct WorldCtx {
  odegpuBatch B;
  DBuf<float> contact_fb;   // contact-joint feedback of the last step
  // capacities the large-world buffers were made for (nb, persistent joints,
  // contacts), kept while a world's next step fits them
  int lw_nb = 0, lw_njp = 0, lw_ccap = 0;
};

WorldCtx* ctx_create(int device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device) {
    cudaGetLastError();
    fail(ODEGPU_E_CUDA, "no CUDA device available");
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) return nullptr;
  auto* c = new WorldCtx();
  c->B.device = device;
  c->B.n_worlds = 1;
  c->B.warps_per_block = 1;
  for (int k = 0; k < 5; ++k) c->B.kwpb[k] = 1;
  if (cudaStreamCreateWithFlags(&c->B.stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    fail(ODEGPU_E_CUDA, "stream creation failed");
    return nullptr;
  }
  configure_kernels();
  return c;
}

void ctx_destroy(WorldCtx* c) {
  if (!c) return;
  cudaSetDevice(c->B.device);
  cudaStreamSynchronize(c->B.stream);
  cudaStreamDestroy(c->B.stream);
  c->B.stream = nullptr;
  delete c;
}

// Uploads of the body, joint and contact arrays shared by both step paths.
static int ctx_upload(odegpuBatch& B, const HostWorld& hw, const WorldDesc& D) {
  cudaStream_t s = B.stream;
  const int nb = D.nb;
  std::vector<WorldDesc> wd(1, D);
  int rc = 0;
  rc = rc ? rc : put(B.world, wd, s);
  rc = rc ? rc : put(B.seed, std::vector<unsigned>(1, hw.seed), s);
  rc = rc ? rc : put(B.status, std::vector<int>(1, 0), s);
  rc = rc ? rc : put(B.ncontacts, std::vector<int>(1, (int)hw.contacts.size()), s);
  rc = rc ? rc : grow(B.nrows, 1);
  rc = rc ? rc : grow(B.nislands, 1);
  rc = rc ? rc : put(B.pos, hw.pos, s);
  rc = rc ? rc : put(B.q, hw.q, s);
  rc = rc ? rc : put(B.lvel, hw.lvel, s);
  rc = rc ? rc : put(B.avel, hw.avel, s);
  rc = rc ? rc : put(B.facc, hw.facc, s);
  rc = rc ? rc : put(B.tacc, hw.tacc, s);
  rc = rc ? rc : put(B.mass, hw.mass, s);
  rc = rc ? rc : put(B.invMass, hw.invMass, s);
  rc = rc ? rc : put(B.I, hw.I, s);
  rc = rc ? rc : put(B.invI, hw.invI, s);
  rc = rc ? rc : grow(B.invIw, 12 * (size_t)nb);
  rc = rc ? rc : put(B.bflags, hw.flags, s);
  B.bstep_on = !hw.bstep.empty();
  if (B.bstep_on) rc = rc ? rc : put(B.bstep, hw.bstep, s);
  rc = rc ? rc : put(B.joints, hw.joints, s);
  rc = rc ? rc : put(B.contacts, hw.contacts, s, (size_t)D.contact_cap);
  rc = rc ? rc : put(B.surfaces, hw.surfaces, s);
  rc = rc ? rc : put(B.padj_start, hw.padj_start, s);
  rc = rc ? rc : put(B.padj, hw.padj, s);
  rc = rc ? rc : grow(B.rows, (size_t)D.row_cap * kRowWords);
  return rc;
}

static int ctx_download(odegpuBatch& B, HostWorld& hw) {
  cudaStream_t s = B.stream;
  const int nb = hw.desc.nb;
  std::vector<int> st(1);
  OG_CUDA(cudaMemcpyAsync(hw.pos.data(), B.pos.p, nb * sizeof(float4), cudaMemcpyDeviceToHost, s));
  OG_CUDA(cudaMemcpyAsync(hw.q.data(), B.q.p, nb * sizeof(float4), cudaMemcpyDeviceToHost, s));
  OG_CUDA(cudaMemcpyAsync(hw.lvel.data(), B.lvel.p, nb * sizeof(float4), cudaMemcpyDeviceToHost, s));
  OG_CUDA(cudaMemcpyAsync(hw.avel.data(), B.avel.p, nb * sizeof(float4), cudaMemcpyDeviceToHost, s));
  OG_CUDA(cudaMemcpyAsync(&hw.seed, B.seed.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  OG_CUDA(cudaMemcpyAsync(st.data(), B.status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  OG_CUDA(cudaStreamSynchronize(s));
  hw.status = st[0];
  return 0;
}

// A world above the on-chip limits (more than 64 bodies, or joints and
// contacts that may need more than 1024 rows) steps through the large-world
// pipeline with the host's contacts and joint lists: no collision, one world.
static int ctx_step_large(WorldCtx* c, HostWorld& hw) {
  odegpuBatch& B = c->B;
  const int nb = hw.desc.nb;
  if (nb > ODEGPU_MAX_BODIES_LARGE)
    return fail(ODEGPU_E_LIMIT, "world has " + std::to_string(nb) + " bodies; at most " +
                                    std::to_string(ODEGPU_MAX_BODIES_LARGE));
  if (hw.exact) return fail(ODEGPU_E_ARG, "dWorldStep is not available for a world above 64 bodies or 1024 rows");
  WorldDesc D = hw.desc;
  D.body_off = D.geom_off = D.joint_off = D.contact_off = D.row_off = D.padj_off = 0;
  D.ng = 0;
  D.fwd_scratch = -1;
  const int nc = (int)hw.contacts.size();
  const bool fits = B.lw && c->lw_nb == nb && c->lw_njp == D.njp && c->lw_ccap >= nc;
  D.contact_cap = fits ? c->lw_ccap : std::max(64, nc + nc / 2);
  D.row_cap = 3 * D.contact_cap + 6 * D.njp;
  B.nb_total = nb;
  B.nj_total = D.njp;
  if (int rc = ctx_upload(B, hw, D)) return rc;
  B.n_ctrl_steps = 0;
  B.feedback_on = false;
  B.exact = false;
  B.n_worlds = 1;
  B.h_world.assign(1, D);
  if (!fits) {
    delete B.lw;
    B.lw = new LargeWorld();
    c->lw_nb = c->lw_njp = c->lw_ccap = 0;
    if (int rc = ::lw_setup(&B, nullptr)) {
      delete B.lw;
      B.lw = nullptr;
      return rc;
    }
    c->lw_nb = nb; c->lw_njp = D.njp; c->lw_ccap = D.contact_cap;
  }
  StepOptions opt{0, nullptr, nullptr, nullptr, 1, 1};
  if (hw.want_feedback) {
    int rc = grow(B.jcopy, (size_t)D.row_cap * 12);
    rc = rc ? rc : grow(B.feedback, (size_t)std::max(1, D.njp) * 12);
    rc = rc ? rc : grow(c->contact_fb, (size_t)std::max(1, D.contact_cap) * 12);
    if (rc) return rc;
    opt.jcopy = B.jcopy.p;
    opt.feedback = B.feedback.p;
    opt.contact_feedback = c->contact_fb.p;
  }
  if (int e = B.launch(0, 1, 1, opt, false)) return e;
  if (hw.want_feedback) {
    hw.feedback.resize((size_t)D.njp * 12);
    hw.contact_feedback.resize((size_t)nc * 12);
    if (!hw.feedback.empty())
      OG_CUDA(cudaMemcpyAsync(hw.feedback.data(), B.feedback.p, hw.feedback.size() * sizeof(float),
                              cudaMemcpyDeviceToHost, B.stream));
    if (!hw.contact_feedback.empty())
      OG_CUDA(cudaMemcpyAsync(hw.contact_feedback.data(), c->contact_fb.p,
                              hw.contact_feedback.size() * sizeof(float), cudaMemcpyDeviceToHost, B.stream));
  }
  return ctx_download(B, hw);
}

int ctx_step(WorldCtx* c, HostWorld& hw) {
  odegpuBatch& B = c->B;
  OG_CUDA(cudaSetDevice(B.device));
  cudaStream_t s = B.stream;
  const int nb = hw.desc.nb;
  if (nb > kMaxB || 6LL * hw.desc.njp + 3LL * (long long)hw.contacts.size() > ODEGPU_MAX_ROWS_PER_WORLD)
    return ctx_step_large(c, hw);
  if (B.lw) {
    delete B.lw;
    B.lw = nullptr;
    c->lw_nb = c->lw_njp = c->lw_ccap = 0;
  }
  B.nb_total = nb;
  B.nj_total = hw.desc.njp;
  WorldDesc D = hw.desc;
  D.body_off = D.geom_off = D.joint_off = D.contact_off = D.row_off = D.padj_off = 0;
  D.ng = 0;
  D.fwd_scratch = D.row_cap > kFwdRows ? 0 : -1;
  const size_t jl = (size_t)D.njp + D.contact_cap;
  int rc = ctx_upload(B, hw, D);
  rc = rc ? rc : grow(B.sweep, ((size_t)D.row_cap + 32) * 8);
  if (D.fwd_scratch >= 0) rc = rc ? rc : grow(B.fwd_scratch, (size_t)kFwdScratchPerWorld);
  rc = rc ? rc : grow(B.jlist, jl);
  rc = rc ? rc : grow(B.jrow, jl);
  rc = rc ? rc : grow(B.jm, jl);
  rc = rc ? rc : grow(B.adj, 2 * jl);
  rc = rc ? rc : grow(B.adj_start, (size_t)nb + 1);
  rc = rc ? rc : grow(B.island_jstart, (size_t)nb + 1);
  rc = rc ? rc : grow(B.island_rstart, (size_t)nb + 1);
  if (rc) return rc;
  B.n_ctrl_steps = 0;
  StepOptions opt{0, nullptr, nullptr, nullptr, 1, 1};
  B.feedback_on = false;
  if (hw.want_feedback) {
    rc = rc ? rc : grow(B.jcopy, (size_t)D.row_cap * 12);
    rc = rc ? rc : grow(B.feedback, (size_t)std::max(1, D.njp) * 12);
    rc = rc ? rc : grow(c->contact_fb, (size_t)std::max(1, D.contact_cap) * 12);
    if (rc) return rc;
    opt.jcopy = B.jcopy.p;
    opt.feedback = B.feedback.p;
    opt.contact_feedback = c->contact_fb.p;
  }
  B.exact = hw.exact;
  B.n_worlds = 1;
  B.h_world.assign(1, D);
  if (int e = B.launch(0, 1, 1, opt, false)) return e;
  if (hw.want_feedback) {
    hw.feedback.resize((size_t)D.njp * 12);
    hw.contact_feedback.resize((size_t)D.contact_cap * 12);
    if (!hw.feedback.empty())
      OG_CUDA(cudaMemcpyAsync(hw.feedback.data(), B.feedback.p, hw.feedback.size() * sizeof(float),
                              cudaMemcpyDeviceToHost, s));
    if (!hw.contact_feedback.empty())
      OG_CUDA(cudaMemcpyAsync(hw.contact_feedback.data(), c->contact_fb.p,
                              hw.contact_feedback.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
  }
  return ctx_download(B, hw);
}

DevHeightfield make_dev_heightfield(int nx, int nz, double width, double depth, double scale, double offset,
                                   double thickness, int wrap, const double* pos, const double* R9, int h_off) {
  DevHeightfield D;
  D.nx = nx; D.nz = nz; D.wrap = wrap; D.h_off = h_off;
  D.width = (float)width; D.depth = (float)depth;
  D.scale = (float)scale; D.offset = (float)offset; D.thickness = (float)thickness;
  const double sw = width / (nx - 1.0), sd = depth / (nz - 1.0);
  D.sw = (float)sw; D.sd = (float)sd;
  D.inv_sw = (float)(1.0 / sw); D.inv_sd = (float)(1.0 / sd);
  D.zx = (float)(sd / sw);
  D.half_w = (float)(width / 2.0); D.half_d = (float)(depth / 2.0);
  for (int k = 0; k < 3; ++k) D.pos[k] = (float)pos[k];
  D.pad = 0.f;
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) D.R[r * 4 + c] = (float)R9[r * 3 + c];
    D.R[r * 4 + 3] = 0.f;
  }
  return D;
}

__global__ void collide_hf_kernel(DevHeightfield H, const float* heights, GeomView g, unsigned flags, Contact* out,
                                  int* n, HFBig big) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    Contact c[8];
    int k = collide_heightfield(H, heights, g, flags, c, nullptr, big);
    if (k < 0) k = -1;
    for (int i = 0; i < k; ++i) out[i] = c[i];
    *n = k;
  }
}

int upload_heights(const std::vector<float>& h, float** dev) {
  if (*dev) { cudaFree(*dev); *dev = nullptr; }
  if (h.empty()) return 0;
  if (cudaMalloc(dev, h.size() * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    *dev = nullptr;
    return fail(ODEGPU_E_NOMEM, "heightfield upload");
  }
  if (cudaMemcpy(*dev, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(ODEGPU_E_CUDA, "heightfield upload");
  return 0;
}

void free_heights(float* dev) {
  if (dev) cudaFree(dev);
}

// dCollide(heightfield, g): the zone in the thread's arrays, or, when the geom
// covers more samples than they hold, in a workspace allocated for the call
// (up to kHFBigZone samples per axis).
int collide_hf_gpu(const DevHeightfield& H, const float* d_heights, const GeomView& g, unsigned flags, Contact* out) {
  const double gp[4] = {g.p[0], g.p[1], g.p[2], g.p[3]};
  const int side = hf_zone_side(aabb_half_bound(g.type, gp), std::min(H.sw, H.sd));
  HFBig big{nullptr, 0};
  if (side > kHFZone) {
    big.side = std::min(side, kHFBigZone);
    OG_CUDA(cudaMalloc(&big.ws, (size_t)hf_ws_bytes(big.side)));
  }
  Contact* d_c = nullptr;
  if (cudaMalloc(&d_c, 8 * sizeof(Contact) + sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    if (big.ws) cudaFree(big.ws);
    return fail(ODEGPU_E_NOMEM, "dCollide staging allocation failed");
  }
  int* d_n = reinterpret_cast<int*>(d_c + 8);
  collide_hf_kernel<<<1, 32>>>(H, d_heights, g, flags, d_c, d_n, big);
  int n = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(&n, d_n, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && n > 0) e = cudaMemcpy(out, d_c, n * sizeof(Contact), cudaMemcpyDeviceToHost);
  cudaFree(d_c);
  if (big.ws) cudaFree(big.ws);
  if (e != cudaSuccess) return fail(ODEGPU_E_CUDA, cudaGetErrorString(e));
  if (n < 0)
    return fail(ODEGPU_E_LIMIT, "the geom covers more than " + std::to_string(kHFBigZone) + " x " +
                                    std::to_string(kHFBigZone) + " heightfield samples");
  return n;
}

// dClosestLineSegmentPoints for the ODE API: the colliders' own routine, run
// on the host (it is __host__ __device__)
void closest_segment_points_host(const float* a1, const float* a2, const float* b1, const float* b2, float* cp1,
                                 float* cp2) {
  closest_segment_points(a1, a2, b1, b2, cp1, cp2);
}

// dBoxBox for the ODE API: the box-box collider run on the host (it is
// __host__ __device__), with its normal, depth and code
int box_box_host(const float* p1, const float* R1, const float* side1, const float* p2, const float* R2,
                 const float* side2, float* normal, float* depth, int* code, unsigned flags, Contact* out) {
  return box_box(p1, R1, side1, p2, R2, side2, normal, flags, out, depth, code);
}

int collide_pair_gpu(const GeomView& a, const GeomView& b, unsigned flags, Contact* out) {
  Contact* d_c = nullptr;
  int* d_n = nullptr;
  OG_CUDA(cudaMalloc(&d_c, 8 * sizeof(Contact) + sizeof(int)));
  d_n = reinterpret_cast<int*>(d_c + 8);
  collide_pair_kernel<<<1, 32>>>(a, b, flags, d_c, d_n);
  int n = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(&n, d_n, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && n > 0) e = cudaMemcpy(out, d_c, n * sizeof(Contact), cudaMemcpyDeviceToHost);
  cudaFree(d_c);
  if (e != cudaSuccess) return fail(ODEGPU_E_CUDA, cudaGetErrorString(e));
  return n;
}

}  // namespace og

// ---------------------------------------------------------------------------
// dCollide without any device allocation (odegpuCollideNoAlloc).
//
// Some hosts cannot call cudaMalloc at the point where they need a contact
// query: an engine that hands all device memory to its own pool allocator, a
// real-time control loop where allocation is forbidden, or a plugin running
// while its host holds the device's memory budget. For them the staging buffer
// the collider writes into lives in this file-scope device array instead of a
// per-call cudaMalloc. Every GPU that loads the library holds it until exit.

namespace {

struct NoAllocScratch {
  og::Contact contacts[ODEGPU_NOALLOC_MAX_CONTACTS];
  int count;
};
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch[1];

__global__ void collide_pair_noalloc_kernel(GeomView a, GeomView b, unsigned flags, NoAllocScratch* s) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    Contact c[8];
    s->count = 0;   // the array keeps the previous call's contents; reset first
    const int k = collide_primitive(a, b, flags, c);
    for (int i = 0; i < k; ++i) s->contacts[i] = c[i];
    s->count = k;
  }
}

GeomView make_view(int cls, const float* p, const float* pos, const float* R) {
  GeomView v;
  v.type = cls;
  for (int k = 0; k < 4; ++k) v.p[k] = p[k];
  for (int k = 0; k < 3; ++k) v.pos[k] = pos ? pos[k] : 0.f;
  for (int k = 0; k < 12; ++k) v.R[k] = R ? R[k] : ((k == 0 || k == 5 || k == 10) ? 1.f : 0.f);
  if (cls == ODEGPU_GEOM_PLANE) {
    // dCreatePlane normalises (ode/src/plane.cpp:40-56)
    float l = v.p[0] * v.p[0] + v.p[1] * v.p[1] + v.p[2] * v.p[2];
    if (l > 0.f) { l = 1.0f / sqrtf(l); for (int k = 0; k < 4; ++k) v.p[k] *= l; }
    else { v.p[0] = 1.f; v.p[1] = v.p[2] = v.p[3] = 0.f; }
  }
  return v;
}

}  // namespace

extern "C" int odegpuCollideNoAlloc(int class1, const float* params1, const float* pos1, const float* R1,
                                    int class2, const float* params2, const float* pos2, const float* R2,
                                    int flags, float* contacts_out) {
  if (!params1 || !params2 || !contacts_out) return fail(ODEGPU_E_ARG, "null argument");
  const int maxc = flags & 0xffff;
  if (maxc < 1) return 0;
  if (maxc > ODEGPU_NOALLOC_MAX_CONTACTS)
    return fail(ODEGPU_E_LIMIT, "odegpuCollideNoAlloc returns at most " +
                                    std::to_string(ODEGPU_NOALLOC_MAX_CONTACTS) + " contacts; asked for " +
                                    std::to_string(maxc));
  for (const int cls : {class1, class2})
    if (cls < ODEGPU_GEOM_SPHERE || cls > ODEGPU_GEOM_RAY)
      return fail(ODEGPU_E_ARG, "odegpuCollideNoAlloc takes sphere, box, capsule, cylinder, plane and ray geoms; "
                                "got class " + std::to_string(cls));
  // Set-up, with the caller's device current: the array's device address in
  // the current context. Host code may not use the symbol's name as an
  // address. The lookup allocates nothing and is repeated on every call
  // rather than cached per device, so a cudaDeviceReset or a host that runs
  // the device under its own context never leaves a stale address behind.
  void* sp = nullptr;
  OG_CUDA(cudaGetSymbolAddress(&sp, g_noalloc_scratch));
  NoAllocScratch* s = static_cast<NoAllocScratch*>(sp);
  const GeomView a = make_view(class1, params1, pos1, R1);
  const GeomView b = make_view(class2, params2, pos2, R2);
  collide_pair_noalloc_kernel<<<1, 32>>>(a, b, (unsigned)flags, s);
  OG_CUDA(cudaGetLastError());
  NoAllocScratch h;
  OG_CUDA(cudaMemcpy(&h, s, sizeof(h), cudaMemcpyDeviceToHost));
  for (int i = 0; i < h.count; ++i) {
    float* o = contacts_out + 7 * i;
    for (int k = 0; k < 3; ++k) { o[k] = h.contacts[i].pos[k]; o[3 + k] = h.contacts[i].normal[k]; }
    o[6] = h.contacts[i].depth;
  }
  return h.count;
}
