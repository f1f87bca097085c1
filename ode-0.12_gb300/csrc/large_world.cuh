// large_world.cuh -- one world of thousands of bodies stepped by the whole
// GPU (the warp-per-world kernels hold a world on chip and stop at 64 bodies).
//
// The step keeps the reference's results and order:
//   * controls, world-frame inertia, gyroscopic torque, gravity: a thread per body;
//   * dCollide over the canonical pair list (geoms i < k in index order, the
//     same early-outs and jointed-body test as the small path): geoms on bodies
//     hash into a uniform grid whose cells are at least one bounding-sphere
//     test wide, each geom lists its partners k > i in index order, static
//     geoms get theirs by an ordered compaction, and one thread per pair runs
//     the collider; prefix sums place every contact at its canonical index;
//   * each body's joint list in ODE's order (contacts newest first, then
//     persistent joints newest first), then the island walk of
//     ode/src/util.cpp:384-521 by one warp;
//   * getInfo1/getInfo2 per joint in island order with the ball / fixed erp
//     carried along each island, rows set up per row;
//   * SOR_LCP (quickstep.cpp:405-583): the findex tail reversal and ODE's
//     Fisher-Yates reshuffle every 8 iterations, computed exactly in parallel
//     (see lw_permute_kernel), then the sweep in that sequential order run as
//     dataflow in one thread-block cluster: every body's velocity accumulator
//     and a counter of the row updates it has received live in distributed
//     shared memory, and a row waits (bounded) until both of its bodies have
//     received exactly the updates that precede it in the order;
//   * integration per body.
#pragma once
#include <cooperative_groups.h>
#include "world_solve.cuh"

namespace og {

constexpr int kLwPartners = 64;        // candidate partners (k > i) one geom may own
constexpr int kLwSweepThreads = 512;   // threads per CTA of the sweep cluster
constexpr int kLwScanThreads = 1024;
constexpr unsigned kLwSpinLimit = 1u << 22;

// One body's slot in the sweep cluster's shared memory.
struct __align__(16) LwBody {
  float f[6];        // constraint force accumulator (cforce)
  unsigned cnt;      // row updates applied to the body in this sweep launch
  int lvl;           // dependency level of the last row that updated it (first iteration)
};
constexpr int kLwLevels = 2048;        // levels the sweep sorts by (more: position order)
constexpr int kLwLevelWindow = 8;      // positions per thread polled together for their levels

struct LWDev {
  int nb, ng, njp, nstat, contact_cap, row_cap, pair_cap, adj_cap, hsize, cluster;
  float cell, inv_cell;
  const int* statics;    // [nstat] static geoms (world-local), ascending
  // broadphase
  int* ghash;            // [ng] bucket of each geom on a body, -1 for static geoms
  int* hcount;           // [hsize+1] geoms per bucket -> first slot
  int* hfill;            // [hsize]
  int* hgeoms;           // [ng]
  int* plist;            // [ng][kLwPartners] partners k > i of geoms on bodies, ascending
  int* pcnt;             // [ng] number of those partners
  int* own;              // [ng+1] pairs owned by each geom -> first pair
  int* sflag;            // [nstat][ng+1] geom k (> s) pairs with static s -> rank
  int* pair_i;           // [pair_cap]
  int* pair_k;           // [pair_cap]
  int* npairs;           // [1]
  int* pnc;              // [pair_cap+1] contacts per pair -> first contact
  Contact* staged;       // [pair_cap][max_contacts]
  // body joint lists
  int* ccount;           // [nb] contacts per body
  int* acount;           // [nb+1] list length -> first entry
  int* afill;            // [nb]
  int* adj_joint;        // [adj_cap] joint ordinal of each entry (persistent j, contact njp + c)
  int* adj_other;        // [adj_cap] the other body of each entry, -1 for none
  // islands
  int* jentry;           // [njp+contact_cap] island order as list entries
  int* jlist;            // [njp+contact_cap] island order as joint ordinals
  int* istart;           // [nb+1] first island-order position of each island with joints
  int* nj;               // [1] joints taken into islands
  int* stack;            // [nb] walk stack when the walk's arrays do not fit on chip
  unsigned char* bflag;  // [nb] walk flags when they do not fit on chip
  // rows
  int* jm;               // [njp+contact_cap+1] rows per island-ordered joint -> first row
  int* bfk;              // [njp+contact_cap] position of a ball / fixed joint, else -1 -> running max
  int* rstart;           // [nb+1] first row of each island
  float* tmp1;           // [nb][6]
  // SOR
  int* rowisl;           // [row_cap] island of each row
  int* neg;              // [row_cap+1] findex == -1 flags -> exclusive scan
  int* draws;            // [nb+1] reshuffle draws of each island -> first draw
  int* order;            // [row_cap] position -> row (two buffers)
  int* order2;
  int* rnd;              // [row_cap] swap partner of each position's reshuffle step
  int* tcount;           // [row_cap+1] steps that swap with each position -> first
  int* tfill;            // [row_cap]
  int* tlist;            // [row_cap]
  int* bcount;           // [nb+1] positions touching each body -> first
  int* bfill;            // [nb]
  int* blist;            // [2*row_cap]
  int4* prec;            // [row_cap] per position: row, rank1 << 16 | deg1, rank2 << 16 | deg2
  int* plev;             // [row_cap] dependency level of each position in the round's order
  int2* ppred;           // [row_cap] previous position on the row's body 1 / body 2 (-1: none)
  float* rsort;          // [row_cap][32] the round's rows in level order (word 31: row index)
  int* lorder;           // [row_cap] positions sorted by level
  float* lambda;         // [row_cap]
  float* fc;             // [nb][6]
  int* err;              // [1] a sweep wait gave up
  unsigned long long* stats;  // [9] diagnostics, see odegpuBatchLargeWorldStats
};

// Diagnostics accumulated on the device (nanoseconds from the global timer).
enum { LWS_WALK_NS = 0, LWS_SWEEP_FIRST_NS = 1, LWS_SWEEP_SORT_NS = 2, LWS_SWEEP_REST_NS = 3,
       LWS_LEVELS_MAX = 4, LWS_SWEEPS = 5, LWS_WALKS = 6, LWS_WALK_COPY_NS = 7, LWS_CLUSTER = 8 };
OG_D unsigned long long lw_now() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// ---------------------------------------------------------------- scans
// In-place exclusive prefix sum of a[0..n) (row blockIdx.x of stride `stride`),
// total in a[n]; n from n_dev when given. One block per row.
__global__ void __launch_bounds__(kLwScanThreads) lw_scan_kernel(int* a, const int* n_dev, int n_host,
                                                                 size_t stride) {
  __shared__ int wsum[32];
  a += (size_t)blockIdx.x * stride;
  const int n = n_dev ? *n_dev : n_host;
  const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int per = (n + T - 1) / T;
  const int s = min(n, tid * per), e = min(n, s + per);
  int sum = 0;
  for (int i = s; i < e; ++i) sum += a[i];
  const int incl = warp_incl_scan(sum, lane);
  if (lane == 31) wsum[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    const int v = (lane < (T >> 5)) ? wsum[lane] : 0;
    const int wi = warp_incl_scan(v, lane);
    wsum[lane] = wi;
  }
  __syncthreads();
  int run = (wid > 0 ? wsum[wid - 1] : 0) + incl - sum;
  for (int i = s; i < e; ++i) {
    const int v = a[i];
    a[i] = run;
    run += v;
  }
  if (tid == 0) a[n] = wsum[(T >> 5) - 1];
}

// In-place inclusive running maximum of a[0..n), n from n_dev.
__global__ void __launch_bounds__(kLwScanThreads) lw_max_scan_kernel(int* a, const int* n_dev) {
  __shared__ int wmax[32];
  const int n = *n_dev;
  const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int per = (n + T - 1) / T;
  const int s = min(n, tid * per), e = min(n, s + per);
  int m = -1;
  for (int i = s; i < e; ++i) m = max(m, a[i]);
  // inclusive max-scan across threads
  int incl = m;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl = max(incl, v);
  }
  if (lane == 31) wmax[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int v = (lane < (T >> 5)) ? wmax[lane] : -1;
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(kFull, v, o);
      if (lane >= o) v = max(v, u);
    }
    wmax[lane] = v;
  }
  __syncthreads();
  int excl = __shfl_up_sync(kFull, incl, 1);
  if (lane == 0) excl = -1;
  int run = max(wid > 0 ? wmax[wid - 1] : -1, excl);
  for (int i = s; i < e; ++i) {
    run = max(run, a[i]);
    a[i] = run;
  }
}

// ---------------------------------------------------------------- bodies
__global__ void lw_bodies_pre_kernel(BatchDev d, int step, int controls, int prologue) {
  const WorldDesc D = d.world[0];
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= D.nb) return;
  if (controls) controls_body(d, step, D.body_off + b);
  if (prologue) body_prologue(d, D, D.body_off + b);
}
__global__ void lw_controls_joints_kernel(BatchDev d, int step) {
  if (threadIdx.x == 0 && blockIdx.x == 0) controls_joints(d, d.world[0], step);
}

// ---------------------------------------------------------------- broadphase
OG_D int lw_cell_hash(int ix, int iy, int iz, int mask) {
  unsigned h = (unsigned)ix * 73856093u ^ (unsigned)iy * 19349663u ^ (unsigned)iz * 83492791u;
  return (int)(h & (unsigned)mask);
}
OG_D void lw_cell_of(const LWDev& L, const float4& p, int& ix, int& iy, int& iz) {
  ix = (int)floorf(p.x * L.inv_cell);
  iy = (int)floorf(p.y * L.inv_cell);
  iz = (int)floorf(p.z * L.inv_cell);
}

__global__ void lw_hash_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= L.ng) return;
  const int b = d.gbody[D.geom_off + g];
  if (b < 0) { L.ghash[g] = -1; return; }
  int ix, iy, iz;
  lw_cell_of(L, d.pos[D.body_off + b], ix, iy, iz);
  const int h = lw_cell_hash(ix, iy, iz, L.hsize - 1);
  L.ghash[g] = h;
  atomicAdd(&L.hcount[h], 1);
}

__global__ void lw_hfill_kernel(LWDev L) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= L.ng) return;
  const int h = L.ghash[g];
  if (h < 0) return;
  const int slot = atomicAdd(&L.hfill[h], 1);
  L.hgeoms[L.hcount[h] + slot] = g;
}

// Could geom g (on a body, bounding radius r at p) touch static geom s? Planes
// are culled by the signed distance of the bounding sphere with the margin of
// the pair pre-test; other static geoms are always candidates.
OG_D bool lw_static_candidate(const BatchDev& d, const WorldDesc& D, int s, const float4& p, float r) {
  const int gs = D.geom_off + s;
  if (d.gtype[gs] != G_PLANE || !isfinite(r)) return true;
  const float4 pl = d.gparam[gs];
  const float dist = pl.x * p.x + pl.y * p.y + pl.z * p.z - pl.w;
  return dist <= r * 1.001f + 1e-5f;
}

// Per geom i on a body: its partners k > i (statics after it, and geoms on
// other bodies within the pair pre-test, not jointed to it), ascending, and
// the flags of the statics before it that pair with it.
__global__ void lw_candidates_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.ng) return;
  const int gi = D.geom_off + i;
  const int bi = d.gbody[gi];
  if (bi < 0) { L.pcnt[i] = 0; L.own[i] = 0; return; }
  const float4 pi4 = d.pos[D.body_off + bi];
  const float ri = d.gbound[gi];
  int* out = L.plist + (size_t)i * kLwPartners;
  int n = 0;
  bool over = false;
  for (int si = 0; si < L.nstat; ++si) {
    const int s = L.statics[si];
    if (!lw_static_candidate(d, D, s, pi4, ri)) continue;
    if (s > i) {
      if (n < kLwPartners) out[n++] = s; else over = true;
    } else {
      L.sflag[(size_t)si * (L.ng + 1) + i] = 1;
    }
  }
  int ix, iy, iz;
  lw_cell_of(L, pi4, ix, iy, iz);
  int buckets[27];
  int nbk = 0;
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz) {
        const int h = lw_cell_hash(ix + dx, iy + dy, iz + dz, L.hsize - 1);
        bool seen = false;
        for (int q = 0; q < nbk; ++q) seen |= (buckets[q] == h);
        if (!seen) buckets[nbk++] = h;
      }
  for (int q = 0; q < nbk; ++q) {
    const int h = buckets[q];
    for (int e = L.hcount[h]; e < L.hcount[h + 1]; ++e) {
      const int k = L.hgeoms[e];
      if (k <= i) continue;
      const int gk = D.geom_off + k;
      const int bk = d.gbody[gk];
      if (bk == bi) continue;
      const float rk = d.gbound[gk];
      if (isfinite(ri) && isfinite(rk)) {
        const float4 pk4 = d.pos[D.body_off + bk];
        const float dx = pi4.x - pk4.x, dy = pi4.y - pk4.y, dz = pi4.z - pk4.z;
        const float lim = (ri + rk) * 1.001f + 1e-5f;
        if (dx * dx + dy * dy + dz * dz > lim * lim) continue;
      }
      if (jointed(d, D, 0, bi, bk)) continue;
      if (n < kLwPartners) out[n++] = k; else over = true;
    }
  }
  // ascending partner order (the canonical pair order within this owner)
  for (int a = 1; a < n; ++a) {
    const int v = out[a];
    int b = a - 1;
    while (b >= 0 && out[b] > v) { out[b + 1] = out[b]; --b; }
    out[b + 1] = v;
  }
  if (over) atomicOr(&d.status[0], ST_PAIR_OVERFLOW);
  L.pcnt[i] = n;
  L.own[i] = n;
}

__global__ void lw_static_own_kernel(LWDev L) {
  const int si = blockIdx.x * blockDim.x + threadIdx.x;
  if (si >= L.nstat) return;
  L.own[L.statics[si]] = L.sflag[(size_t)si * (L.ng + 1) + L.ng];
}

__global__ void lw_pairs_fill_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0) {
    const int total = L.own[L.ng];
    if (total > L.pair_cap) atomicOr(&d.status[0], ST_PAIR_OVERFLOW);
    *L.npairs = min(total, L.pair_cap);
  }
  if (k >= L.ng || d.gbody[D.geom_off + k] < 0) return;
  const int* in = L.plist + (size_t)k * kLwPartners;
  const int base = L.own[k];
  for (int j = 0; j < L.pcnt[k]; ++j) {
    const int pos = base + j;
    if (pos < L.pair_cap) { L.pair_i[pos] = k; L.pair_k[pos] = in[j]; }
  }
  for (int si = 0; si < L.nstat; ++si) {
    const int s = L.statics[si];
    if (s >= k) break;
    const int* f = L.sflag + (size_t)si * (L.ng + 1);
    if (f[k + 1] == f[k]) continue;
    const int pos = L.own[s] + f[k];
    if (pos < L.pair_cap) { L.pair_i[pos] = s; L.pair_k[pos] = k; }
  }
}

// dCollide(g_i, g_k) of every candidate pair into its staging slots.
__global__ void __launch_bounds__(128) lw_narrow_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = *L.npairs;
  if (p >= np) return;
  const int i = L.pair_i[p], k = L.pair_k[p];
  GeomView vi, vk;
  geom_view(d, D, i, vi);
  geom_view(d, D, k, vk);
  Contact cc[8];
  int cnt = 0;
  if (vi.type == G_HEIGHTFIELD || vk.type == G_HEIGHTFIELD) {
    cnt = collide_hf_pair(d, vi, vk, (unsigned)D.max_contacts, cc, nullptr, HFBig{nullptr, 0});
    if (cnt < 0) {
      // a zone beyond the thread's arrays: lw_hf_big_kernel collides it
      // through the world's workspace (when it has one)
      if (D.hf_ws_side > 0) { L.pnc[p] = -1; return; }
      atomicOr(&d.status[0], ST_HF_ZONE);
      cnt = 0;
    }
  } else {
    cnt = collide_primitive(vi, vk, (unsigned)D.max_contacts, cc);
  }
  Contact* o = L.staged + (size_t)p * D.max_contacts;
  for (int c = 0; c < cnt; ++c) o[c] = cc[c];
  L.pnc[p] = cnt;
}

// The heightfield pairs lw_narrow_kernel left (count -1): one warp finds them
// and collides them one at a time through the world's workspace, which they
// share.
__global__ void __launch_bounds__(32) lw_hf_big_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int lane = threadIdx.x;
  const int np = *L.npairs;
  const HFBig big{d.hf_ws + D.hf_ws, D.hf_ws_side};
  for (int base = 0; base < np; base += 32) {
    const int p = base + lane;
    unsigned todo = __ballot_sync(kFull, p < np && L.pnc[p] < 0);
    while (todo) {
      const int l = __ffs(todo) - 1;
      todo &= todo - 1;
      if (lane == l) {
        GeomView vi, vk;
        geom_view(d, D, L.pair_i[p], vi);
        geom_view(d, D, L.pair_k[p], vk);
        Contact cc[8];
        int cnt = collide_hf_pair(d, vi, vk, (unsigned)D.max_contacts, cc, nullptr, big);
        if (cnt < 0) { atomicOr(&d.status[0], ST_HF_ZONE); cnt = 0; }
        Contact* o = L.staged + (size_t)p * D.max_contacts;
        for (int c = 0; c < cnt; ++c) o[c] = cc[c];
        L.pnc[p] = cnt;
      }
      __syncwarp();
    }
  }
}

// Contact joints in canonical order (dJointCreateContact + dJointAttach(body(g_i), body(g_k))).
__global__ void lw_contacts_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = *L.npairs;
  if (p == 0) {
    const int total = L.pnc[np];
    if (total > L.contact_cap) atomicOr(&d.status[0], ST_CONTACT_OVERFLOW);
    d.ncontacts[0] = min(total, L.contact_cap);
  }
  if (p >= np) return;
  const int n = L.pnc[p + 1] - L.pnc[p];
  if (n == 0) return;
  const int i = L.pair_i[p], k = L.pair_k[p];
  const int bi = d.gbody[D.geom_off + i], bk = d.gbody[D.geom_off + k];
  const int si = d.gsurf[D.geom_off + i], sk = d.gsurf[D.geom_off + k];
  const Contact* in = L.staged + (size_t)p * D.max_contacts;
  for (int c = 0; c < n; ++c) {
    const int slot = L.pnc[p] + c;
    if (slot >= L.contact_cap) break;
    DevContact ct;
    ct.pos[0] = in[c].pos[0]; ct.pos[1] = in[c].pos[1]; ct.pos[2] = in[c].pos[2];
    ct.depth = in[c].depth;
    ct.normal[0] = in[c].normal[0]; ct.normal[1] = in[c].normal[1]; ct.normal[2] = in[c].normal[2];
    ct.surface = si > sk ? si : sk;
    if (bi < 0) { ct.b1 = bk; ct.b2 = -1; ct.reverse = 1; }
    else { ct.b1 = bi; ct.b2 = bk; ct.reverse = 0; }
    ct.geoms = -1;
    d.contacts[D.contact_off + slot] = ct;
    atomicAdd(&L.ccount[ct.b1], 1);
    if (ct.b2 >= 0) atomicAdd(&L.ccount[ct.b2], 1);
  }
}

// ---------------------------------------------------------------- body joint lists
__global__ void lw_adj_count_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= L.nb) return;
  const int* ps = d.padj_start + D.body_off;
  L.acount[b] = L.ccount[b] + (ps[b + 1] - ps[b]);
}

__global__ void lw_adj_fill_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.ncontacts[0]) return;
  const DevContact& ct = d.contacts[D.contact_off + c];
  {
    const int e = L.acount[ct.b1] + atomicAdd(&L.afill[ct.b1], 1);
    L.adj_joint[e] = L.njp + c;
    L.adj_other[e] = ct.b2;
  }
  if (ct.b2 >= 0) {
    const int e = L.acount[ct.b2] + atomicAdd(&L.afill[ct.b2], 1);
    L.adj_joint[e] = L.njp + c;
    L.adj_other[e] = ct.b1;
  }
}

// Each body's list: contacts newest first (dJointAttach prepends), then its
// persistent joints in their stored newest-first order.
__global__ void lw_adj_finish_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= L.nb) return;
  const int s = L.acount[b], nc = L.ccount[b];
  int* J = L.adj_joint + s;
  int* O = L.adj_other + s;
  for (int a = 1; a < nc; ++a) {
    const int vj = J[a], vo = O[a];
    int q = a - 1;
    while (q >= 0 && J[q] < vj) { J[q + 1] = J[q]; O[q + 1] = O[q]; --q; }
    J[q + 1] = vj;
    O[q + 1] = vo;
  }
  // (a host-supplied list may hold contacts too: ordinals njp and up)
  const int* ps = d.padj_start + D.body_off;
  int e = s + nc;
  for (int k = ps[b]; k < ps[b + 1]; ++k, ++e) {
    const int j = d.padj[k];
    int b1, b2;
    if (j < L.njp) {
      const DevJoint& Jt = d.joints[D.joint_off + j];
      b1 = Jt.b1; b2 = Jt.b2;
    } else {
      const DevContact& ct = d.contacts[D.contact_off + j - L.njp];
      b1 = ct.b1; b2 = ct.b2;
    }
    L.adj_joint[e] = j;
    L.adj_other[e] = (b1 == b) ? b2 : b1;
  }
}

// The island walk of ode/src/util.cpp:384-521: bodies from the newest (ODE's
// body list is newest first), each untagged one starting a depth-first walk;
// a body's list entries are taken in order. An entry's joint is still
// untagged exactly when its other body has not been walked yet (a joint is
// tagged when the first of its two bodies is walked), so the walk needs only
// the other body of each entry. Every step depends on the one before, so one
// thread runs it; the pointer types tell the compiler which instance keeps its
// arrays on chip (plain shared-memory accesses) and which in global memory.
// Output: the island order as list entries, and the first position of every
// island that has joints.
template <typename OtherT>
OG_D void lw_walk(const LWDev& L, const int* astart, int* stack, unsigned char* flags, const OtherT* other,
                  int nb, int& jc_out, int& ni_out) {
  int jc = 0, ni = 0;
  for (int bb = nb - 1; bb >= 0; --bb) {
    if (flags[bb] & 5) continue;   // walked, or woken by this step (4): not a start
    flags[bb] = 1;
    const int jstart = jc;
    int sp = 0, b = bb;
    for (;;) {
      const int s0 = astart[b], e0 = astart[b + 1];
      for (int k = s0; k < e0; ++k) {
        const int o = (int)other[k];
        if (o < 0) { L.jentry[jc++] = k; continue; }
        const unsigned char fo = flags[o];
        if (fo & 2) continue;
        L.jentry[jc++] = k;
        if (!(fo & 1)) { flags[o] = (unsigned char)(fo | 1); stack[sp++] = o; }
      }
      flags[b] |= 2;
      if (sp == 0) break;
      b = stack[--sp];
    }
    if (jc > jstart) L.istart[ni++] = jstart;
  }
  jc_out = jc;
  ni_out = ni;
}

__global__ void __launch_bounds__(32) lw_islands_kernel(BatchDev d, LWDev L, int smem_bytes) {
  extern __shared__ __align__(16) unsigned char lw_sm[];
  const int lane = threadIdx.x;
  const unsigned long long t_start = lw_now();
  const int nb = L.nb;
  const int E = L.acount[nb];
  // on chip when they fit: list starts, stack, flags, and the other body of
  // every entry as 16 bits (below 32767 bodies)
  const size_t fixed = (size_t)(nb + 1) * 4 + (size_t)nb * 4 + ((nb + 16) & ~15);
  const bool on_chip = nb < 32767 && fixed + (size_t)E * 2 <= (size_t)smem_bytes;
  int jc = 0, ni = 0;
  if (on_chip) {
    int* astart = reinterpret_cast<int*>(lw_sm);
    int* stack = astart + (nb + 1);
    unsigned char* flags = reinterpret_cast<unsigned char*>(stack + nb);
    short* other = reinterpret_cast<short*>(flags + ((nb + 16) & ~15));
    for (int b = lane; b <= nb; b += 32) astart[b] = L.acount[b];
    for (int e = lane; e < E; e += 32) other[e] = (short)L.adj_other[e];
    for (int b = lane; b < nb; b += 32) flags[b] = (d.bflags[b] & BODY_WOKEN) ? 4 : 0;
    __syncwarp();
    if (lane == 0) {
      atomicAdd(&L.stats[LWS_WALK_COPY_NS], lw_now() - t_start);
      lw_walk<short>(L, astart, stack, flags, other, nb, jc, ni);
    }
  } else {
    for (int b = lane; b < nb; b += 32) L.bflag[b] = (d.bflags[b] & BODY_WOKEN) ? 4 : 0;
    __syncwarp();
    if (lane == 0) lw_walk<int>(L, L.acount, L.stack, L.bflag, L.adj_other, nb, jc, ni);
  }
  if (lane == 0) {
    L.istart[ni] = jc;
    *L.nj = jc;
    d.nislands[0] = ni;
    atomicAdd(&L.stats[LWS_WALK_NS], lw_now() - t_start);
    atomicAdd(&L.stats[LWS_WALKS], 1ull);
  }
}

OG_D int lw_island_of(const int* start, int n, int k) {
  // last island whose first position is <= k
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= k) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------- rows
__global__ void lw_info1_kernel(BatchDev d, LWDev L, int step) {
  const WorldDesc D = d.world[0];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int nj = *L.nj;
  if (k >= nj) return;
  const int ord = L.adj_joint[L.jentry[k]];
  L.jlist[k] = ord;
  int m;
  bool bf = false;
  if (ord < D.njp) {
    const DevJoint& J = d.joints[D.joint_off + ord];
    const DevLimot lm1 = step_limot1(J, step_stops(d, D, step), ord);
    BodyRef B1, B2;
    load_body_ref(d, D.body_off + J.b1, B1);
    if (J.b2 >= 0) load_body_ref(d, D.body_off + J.b2, B2);
    m = persistent_info1(J, lm1, B1, J.b2 >= 0 ? &B2 : nullptr).m;
    bf = J.type == J_BALL || J.type == J_FIXED;
  } else {
    m = contact_info1(d.surfaces[d.contacts[D.contact_off + ord - D.njp].surface]);
  }
  L.jm[k] = m;
  L.bfk[k] = bf ? k : -1;
}

__global__ void lw_info2_kernel(BatchDev d, LWDev L, int step) {
  const WorldDesc D = d.world[0];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int nj = *L.nj;
  const int M = L.jm[nj];
  if (k == 0) {
    if (M > L.row_cap) atomicOr(&d.status[0], ST_ROW_OVERFLOW);
    d.nrows[0] = M > L.row_cap ? 0 : M;
  }
  if (M > L.row_cap || k >= nj) return;
  const int nisl = d.nislands[0];
  const int isl = lw_island_of(L.istart, nisl, k);
  if (k == L.istart[isl]) L.rstart[isl] = L.jm[k];
  if (k == 0) L.rstart[nisl] = M;
  // the erp this joint meets: that of the last ball / fixed joint before it
  // in its island (ball.cpp:59, fixed.cpp:80), else the world's
  float erp = D.erp;
  if (k > 0) {
    const int j = L.bfk[k - 1];
    if (j >= L.istart[isl]) erp = d.joints[D.joint_off + L.jlist[j]].erp;
  }
  assemble_joint_rows(d, D, L.jlist[k], L.jm[k], L.jm[k + 1] - L.jm[k], erp, step_stops(d, D, step), nullptr);
}

__global__ void lw_tmp1_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= L.nb || d.nrows[0] == 0) return;
  body_tmp1(d, D.body_off + b, 1.0f / D.dt, L.tmp1 + 6 * (size_t)b);
}

// jcopy (optional): J of every row before scaling, kept for joint feedback
__global__ void lw_row_setup_kernel(BatchDev d, LWDev L, float* jcopy) {
  const WorldDesc D = d.world[0];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= d.nrows[0]) return;
  row_setup(d, D, r, L.tmp1, 1.0f / D.dt, D.sor_w, nullptr, jcopy);
}

// ---------------------------------------------------------------- SOR order
// Per row: its island and whether findex == -1; per island: its reshuffle draws.
__global__ void lw_order_flags_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int M = d.nrows[0];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int nisl = d.nislands[0];
  if (r < nisl) {
    const int m = L.rstart[r + 1] - L.rstart[r];
    L.draws[r] = m > 0 ? ((D.iterations + 7) / 8) * (m - 1) : 0;
  }
  if (r >= M) return;
  L.rowisl[r] = lw_island_of(L.rstart, nisl, r);
  L.neg[r] = reinterpret_cast<const int*>(d.rows + (size_t)(D.row_off + r) * kRowWords)[kRowFindex] == -1 ? 1 : 0;
}

// quickstep.cpp:405-425: rows with findex == -1 first in row order, the rest
// from the island's tail backwards.
__global__ void lw_order_init_kernel(BatchDev d, LWDev L) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= d.nrows[0]) return;
  const int isl = L.rowisl[r];
  const int rs = L.rstart[isl], re = L.rstart[isl + 1];
  const int negb = L.neg[r] - L.neg[rs];
  const bool is_neg = (L.neg[r + 1] - L.neg[r]) != 0;
  const int p = is_neg ? rs + negb : re - 1 - ((r - rs) - negb);
  L.order[p] = r;
}

// Reshuffle `round` (iteration 8 * round): for island position q >= 1 the
// reference swaps order[q] with order[dRandInt(q + 1)], the q-th draw of the
// island's round (quickstep.cpp:471-478). Record the partner and count, per
// position, the steps that swap with it.
__global__ void lw_rand_kernel(BatchDev d, LWDev L, int round) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.nrows[0]) return;
  const int isl = L.rowisl[p];
  const int rs = L.rstart[isl], m = L.rstart[isl + 1] - rs;
  const int q = p - rs;
  if (q == 0) { L.rnd[p] = -1; return; }
  const unsigned k = (unsigned)L.draws[isl] + (unsigned)(round * (m - 1)) + (unsigned)q;
  const int sw = rand_int_from(lcg_jump(d.seed[0], k), q + 1);
  L.rnd[p] = rs + sw;
  atomicAdd(&L.tcount[rs + sw], 1);
}

__global__ void lw_tfill_kernel(BatchDev d, LWDev L) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.nrows[0]) return;
  const int t = L.rnd[p];
  if (t < 0) return;
  L.tlist[L.tcount[t] + atomicAdd(&L.tfill[t], 1)] = p;
}

__global__ void lw_tsort_kernel(BatchDev d, LWDev L) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.nrows[0]) return;
  int* a = L.tlist + L.tcount[q];
  const int n = L.tcount[q + 1] - L.tcount[q];
  for (int i = 1; i < n; ++i) {
    const int v = a[i];
    int j = i - 1;
    while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; --j; }
    a[j + 1] = v;
  }
}

// The permutation the reshuffle's swap sequence applies, without running it
// in sequence. Step j (1 <= j < m) swaps positions j and r_j <= j, and
// position j is untouched before step j, so step j writes the round's old
// entry j to position r_j. Hence the entry at position q just before step t
// (t > q) is old[j] for the last step j < t with r_j = q (j = q when r_q = q),
// and when there is none, what step q moved there: the entry at position r_q
// just before step q (position 0 keeps old[0]). The final entry at q follows
// this chain down r_q < q (O(log m) links for a uniform draw).
__global__ void lw_permute_kernel(BatchDev d, LWDev L, const int* src_order, int* dst_order) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.nrows[0]) return;
  const int isl = L.rowisl[p];
  const int rs = L.rstart[isl], re = L.rstart[isl + 1];
  int t = re, q = p, src = -1;
  for (int guard = 0; guard <= re - rs; ++guard) {
    const int a = L.tcount[q], b = L.tcount[q + 1];
    int j = -1;
    for (int e = b - 1; e >= a; --e) {
      const int v = L.tlist[e];
      if (v < t) { j = v; break; }
    }
    if (j >= 0) { src = j; break; }
    if (q == rs) { src = rs; break; }
    t = q;
    q = L.rnd[q];
  }
  dst_order[p] = src_order[src >= 0 ? src : p];
}

// Positions touching each body, in order: a body's k-th position waits for k
// of the body's updates in every iteration.
__global__ void lw_bodypos_kernel(BatchDev d, LWDev L, const int* ord) {
  const WorldDesc D = d.world[0];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.nrows[0]) return;
  const int r = ord[p];
  const int* w = reinterpret_cast<const int*>(d.rows + (size_t)(D.row_off + r) * kRowWords);
  L.prec[p].x = r;
  L.ppred[p] = make_int2(-1, -1);
  atomicAdd(&L.bcount[w[kRowB1]], 1);
  if (w[kRowB2] >= 0) atomicAdd(&L.bcount[w[kRowB2]], 1);
}

__global__ void lw_bfill_kernel(BatchDev d, LWDev L, const int* ord) {
  const WorldDesc D = d.world[0];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.nrows[0]) return;
  const int* w = reinterpret_cast<const int*>(d.rows + (size_t)(D.row_off + ord[p]) * kRowWords);
  const int b1 = w[kRowB1], b2 = w[kRowB2];
  L.blist[L.bcount[b1] + atomicAdd(&L.bfill[b1], 1)] = p;
  if (b2 >= 0) L.blist[L.bcount[b2] + atomicAdd(&L.bfill[b2], 1)] = p;
}

__global__ void lw_branks_kernel(BatchDev d, LWDev L, const int* ord) {
  const WorldDesc D = d.world[0];
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= L.nb) return;
  int* a = L.blist + L.bcount[b];
  const int n = L.bcount[b + 1] - L.bcount[b];
  if (n >= 65536) { atomicOr(&d.status[0], ST_ROW_OVERFLOW); return; }
  for (int i = 1; i < n; ++i) {
    const int v = a[i];
    int j = i - 1;
    while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; --j; }
    a[j + 1] = v;
  }
  for (int i = 0; i < n; ++i) {
    const int p = a[i];
    const int* w = reinterpret_cast<const int*>(d.rows + (size_t)(D.row_off + ord[p]) * kRowWords);
    const int v = (i << 16) | n;
    const int pred = i > 0 ? a[i - 1] : -1;
    if (w[kRowB1] == b) { L.prec[p].y = v; L.ppred[p].x = pred; }
    else { L.prec[p].z = v; L.ppred[p].y = pred; }
  }
}

// ---------------------------------------------------------------- sweep
OG_D unsigned lw_ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.cluster.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
OG_D void lw_st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.cluster.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Cluster barrier in two halves: work issued between them (a prefetch) is
// not held up by the release, which waits only for what precedes the arrive.
OG_D void lw_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
OG_D void lw_wait_all() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

OG_D int lw_ld_acquire_int(const int* p) {
  int v;
  asm volatile("ld.acquire.cluster.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
OG_D void lw_st_release_int(int* p, int v) {
  asm volatile("st.release.cluster.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Wait (bounded, backing off) until a level is set; false when it gave up.
OG_D bool lw_wait_level(const int* p, int& out, const volatile int* err) {
  unsigned ns = 0;
  for (unsigned spins = 0;; ++spins) {
    const int v = lw_ld_acquire_int(p);
    if (v != 0) { out = v; return true; }
    if (spins >= kLwSpinLimit) return false;
    if ((spins & 255u) == 255u && *err) return false;
    if (spins >= 2) {
      ns = ns ? min(ns * 2u, 256u) : 32u;
      __nanosleep(ns);
    }
  }
}

// Wait until *c == target; false when the wait gave up (bounded, or another
// thread gave up first).
// Polls back off (up to 256 ns apart) so that waiting threads leave the
// cluster's shared-memory network to the rows that are running.
OG_D bool lw_wait(const unsigned* c, unsigned target, const volatile int* err) {
  unsigned ns = 0;
  for (unsigned spins = 0;; ++spins) {
    if (lw_ld_acquire(c) == target) return true;
    if (spins >= kLwSpinLimit) return false;
    if ((spins & 255u) == 255u && *err) return false;
    if (spins >= 2) {
      ns = ns ? min(ns * 2u, 256u) : 32u;
      __nanosleep(ns);
    }
  }
}

// One row update of the sweep (quickstep.cpp:484-582, the arithmetic of
// sor_row term for term) once both bodies have received exactly the updates
// that precede the row: the k-th of deg positions touching a body waits for
// li * deg + k. When lvl_out is given, the row's dependency level (one more
// than the last level recorded on either body) is recorded and passed on.
struct LwRow {
  float4 rw[8];
  int4 rec;
};
OG_D void lw_load(const float* rows, const LWDev& L, int p, LwRow& R) {
  R.rec = L.prec[p];
  load_row(rows, R.rec.x, R.rw);
}
// the j-th row of the round's level order (its row index in word 31)
OG_D void lw_load_sorted(const LWDev& L, int j, LwRow& R) {
  load_row(L.rsort, j, R.rw);
  R.rec = make_int4(__float_as_int(R.rw[7].w), 0, 0, 0);
}
OG_D bool lw_update(cooperative_groups::cluster_group& cluster, int C, LwBody* bodies, float* lam, const LwRow& R,
                    unsigned li, const LWDev& L, int* lvl_out, bool wait = true) {
  const float* J = reinterpret_cast<const float*>(&R.rw[0]);
  const float* iMJ = reinterpret_cast<const float*>(&R.rw[3]);
  const float bb = R.rw[6].x, Ad = R.rw[6].y, lo = R.rw[6].z, hi = R.rw[6].w;
  const int findex = __float_as_int(R.rw[7].x);
  const int b1 = __float_as_int(R.rw[7].y), b2 = __float_as_int(R.rw[7].z);
  const int r = R.rec.x;
  const int lc = __ffs(C) - 1, cm = C - 1;   // C is a power of two
  LwBody* B1 = cluster.map_shared_rank(bodies + (b1 >> lc), b1 & cm);
  LwBody* B2 = b2 >= 0 ? cluster.map_shared_rank(bodies + (b2 >> lc), b2 & cm) : nullptr;
  const unsigned tg1 = li * (unsigned)(R.rec.y & 0xffff) + ((unsigned)R.rec.y >> 16);
  const unsigned tg2 = li * (unsigned)(R.rec.z & 0xffff) + ((unsigned)R.rec.z >> 16);
  if (wait && (!lw_wait(&B1->cnt, tg1, L.err) || (B2 && !lw_wait(&B2->cnt, tg2, L.err)))) {
    atomicExch(L.err, 1);
    return false;
  }
  float* lr = cluster.map_shared_rank(lam + (r >> lc), r & cm);
  const float old = *lr;
  const float lf = findex >= 0 ? *cluster.map_shared_rank(lam + (findex >> lc), findex & cm) : 0.f;
  const float4 a1 = *reinterpret_cast<const float4*>(B1->f);
  const float2 c1 = *reinterpret_cast<const float2*>(B1->f + 4);
  const float f10 = a1.x, f11 = a1.y, f12 = a1.z, f13 = a1.w, f14 = c1.x, f15 = c1.y;
  float f20 = 0.f, f21 = 0.f, f22 = 0.f, f23 = 0.f, f24 = 0.f, f25 = 0.f;
  if (B2) {
    const float4 a2 = *reinterpret_cast<const float4*>(B2->f);
    const float2 c2 = *reinterpret_cast<const float2*>(B2->f + 4);
    f20 = a2.x; f21 = a2.y; f22 = a2.z; f23 = a2.w; f24 = c2.x; f25 = c2.y;
  }
  float delta = bb - old * Ad;
  delta -= (f10 * J[0] + f11 * J[1]) + (f12 * J[2] + f13 * J[3]) + (f14 * J[4] + f15 * J[5]);
  delta -= (f20 * J[6] + f21 * J[7]) + (f22 * J[8] + f23 * J[9]) + (f24 * J[10] + f25 * J[11]);
  const float hf = fabsf(hi * lf);
  const float hi_act = findex >= 0 ? hf : hi;
  const float lo_act = findex >= 0 ? -hf : lo;
  const float nl = old + delta;
  const bool clamped = (nl < lo_act) || (nl > hi_act);
  const float lamv = fminf(fmaxf(nl, lo_act), hi_act);
  delta = clamped ? lamv - old : delta;
  *lr = clamped ? lamv : nl;
  *reinterpret_cast<float4*>(B1->f) =
      make_float4(f10 + delta * iMJ[0], f11 + delta * iMJ[1], f12 + delta * iMJ[2], f13 + delta * iMJ[3]);
  *reinterpret_cast<float2*>(B1->f + 4) = make_float2(f14 + delta * iMJ[4], f15 + delta * iMJ[5]);
  if (lvl_out) {
    const int lv = 1 + max(B1->lvl, B2 ? B2->lvl : 0);
    *lvl_out = lv;
    B1->lvl = lv;
    if (B2) B2->lvl = lv;
  }
  if (B2) {
    *reinterpret_cast<float4*>(B2->f) =
        make_float4(f20 + delta * iMJ[6], f21 + delta * iMJ[7], f22 + delta * iMJ[8], f23 + delta * iMJ[9]);
    *reinterpret_cast<float2*>(B2->f + 4) = make_float2(f24 + delta * iMJ[10], f25 + delta * iMJ[11]);
    if (wait) lw_st_release(&B2->cnt, tg2 + 1u);
  }
  if (wait) lw_st_release(&B1->cnt, tg1 + 1u);
  return true;
}

// Iterations [it0, it1) of SOR_LCP over every island in the current order, as
// one cluster of C = 2^lc CTAs. Body b's slot lives in CTA b & (C-1), row r's
// lambda in CTA r & (C-1).
//   1. Levels: a row's dependency level is one more than the larger level of
//      the previous position on either of its bodies (the per-body position
//      lists give those links); relaxed in parallel passes until no level
//      changes (as many passes as the longest chain).
//   2. Positions counting-sorted by level (per-CTA histograms merged over
//      distributed shared memory).
//   3. Every iteration level by level: the rows of a level touch disjoint
//      bodies and run in parallel, spread over all CTAs; a cluster barrier
//      orders the levels. Each body meets its rows in the sequential order,
//      so the result is the sequential sweep.
// When the levels exceed the histogram the sweep runs in order position as
// dataflow instead: a row waits (bounded) until both bodies have received
// the updates that precede it (the k-th of deg positions touching a body
// waits for it * deg + k).
__global__ void __launch_bounds__(kLwSweepThreads) lw_sweep_kernel(BatchDev d, LWDev L, int it0, int it1,
                                                                   int first) {
  namespace cg = cooperative_groups;
  extern __shared__ __align__(16) unsigned char lw_sw[];
  __shared__ int hist[kLwLevels];       // this CTA's positions per level (read by every CTA)
  __shared__ int ltot[kLwLevels + 1];   // the cluster's positions per level, then each level's first slot
  __shared__ int base[kLwLevels];       // this CTA's next slot of each level
  __shared__ int wsum[32];
  __shared__ int cmax;
  __shared__ int gmax[32];
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int lc = __ffs(C) - 1;
  const int rank = (int)cluster.block_rank();
  const WorldDesc D = d.world[0];
  const int M = d.nrows[0];
  const int nb = L.nb;
  const int nbs = (nb + C - 1) >> lc;
  LwBody* bodies = reinterpret_cast<LwBody*>(lw_sw);
  float* lam = reinterpret_cast<float*>(bodies + nbs);
  const int nrs = (L.row_cap + C - 1) >> lc;
  for (int s = threadIdx.x; s < nbs; s += blockDim.x) {
    const int b = (s << lc) + rank;
    LwBody v;
    for (int k = 0; k < 6; ++k) v.f[k] = (b < nb && !first) ? L.fc[6 * (size_t)b + k] : 0.f;
    v.cnt = 0u;
    v.lvl = 0;
    bodies[s] = v;
  }
  for (int s = threadIdx.x; s < nrs; s += blockDim.x) {
    const int r = (s << lc) + rank;
    lam[s] = (r < M && !first) ? L.lambda[r] : 0.f;
  }
  for (int l = threadIdx.x; l < kLwLevels; l += blockDim.x) hist[l] = 0;
  const int T = C * (int)blockDim.x;
  const int tid = rank * (int)blockDim.x + (int)threadIdx.x;
  const float* rows = d.rows + (size_t)D.row_off * kRowWords;
  const bool timer = rank == 0 && threadIdx.x == 0;
  unsigned long long t_mark = timer ? lw_now() : 0ull;
  // levels live in distributed shared memory next to the lambdas: position p
  // in CTA p & (C-1), 0 until set
  int* lvl = reinterpret_cast<int*>(lam + nrs);
  for (int s = threadIdx.x; s < nrs; s += blockDim.x) lvl[s] = 0;
  if (threadIdx.x == 0) cmax = 0;
  cluster.sync();
  // 1. levels as dataflow: a position takes its level once both predecessors
  //    have theirs. A thread holds up to kLwLevelWindow positions and polls
  //    them in turn, taking whichever is ready, so it never waits behind one
  //    that is not; more positions per thread are taken in order.
  const int lane = tid & 31, wid = tid >> 5, nw = T >> 5;
  const int t0 = lane * nw + wid;
  bool ok = M > 0 && !*L.err;
  {
    int lmax = 0;
    int2 pr[kLwLevelWindow];
    unsigned pending = 0u;
#pragma unroll
    for (int q = 0; q < kLwLevelWindow; ++q) {
      const int p = t0 + q * T;
      pr[q] = p < M ? L.ppred[p] : make_int2(-1, -1);
      if (p < M) pending |= 1u << q;
    }
    unsigned ns = 0;
    for (unsigned spins = 0; ok && pending; ++spins) {
      bool progress = false;
#pragma unroll
      for (int q = 0; q < kLwLevelWindow; ++q) {
        if (!(pending & (1u << q))) continue;
        const int a = pr[q].x, c = pr[q].y;
        const int l1 = a >= 0 ? lw_ld_acquire_int(cluster.map_shared_rank(lvl + (a >> lc), a & (C - 1))) : 1 << 30;
        const int l2 = c >= 0 ? lw_ld_acquire_int(cluster.map_shared_rank(lvl + (c >> lc), c & (C - 1))) : 1 << 30;
        if (l1 == 0 || l2 == 0) continue;
        const int lv = 1 + max(a >= 0 ? l1 : 0, c >= 0 ? l2 : 0);
        const int p = t0 + q * T;
        lw_st_release_int(cluster.map_shared_rank(lvl + (p >> lc), p & (C - 1)), lv);
        lmax = max(lmax, lv);
        pending &= ~(1u << q);
        progress = true;
      }
      if (progress) { ns = 0; continue; }
      if (spins >= kLwSpinLimit || ((spins & 255u) == 255u && *L.err)) { atomicExch(L.err, 1); ok = false; break; }
      ns = ns ? min(ns * 2u, 256u) : 32u;
      __nanosleep(ns);
    }
    for (int p = t0 + kLwLevelWindow * T; ok && p < M; p += T) {
      const int2 pp = L.ppred[p];
      int l1 = 0, l2 = 0;
      if ((pp.x >= 0 && !lw_wait_level(cluster.map_shared_rank(lvl + (pp.x >> lc), pp.x & (C - 1)), l1, L.err)) ||
          (pp.y >= 0 && !lw_wait_level(cluster.map_shared_rank(lvl + (pp.y >> lc), pp.y & (C - 1)), l2, L.err))) {
        atomicExch(L.err, 1);
        ok = false;
        break;
      }
      const int lv = 1 + max(l1, l2);
      lw_st_release_int(cluster.map_shared_rank(lvl + (p >> lc), p & (C - 1)), lv);
      lmax = max(lmax, lv);
    }
    atomicMax(&cmax, lmax);
  }
  cluster.sync();
  if ((int)threadIdx.x < C) gmax[threadIdx.x] = *cluster.map_shared_rank(&cmax, (int)threadIdx.x);
  cluster.sync();
  int nlev = 0;
  for (int c = 0; c < C; ++c) nlev = max(nlev, gmax[c]);
  // every thread reads the flag here, two barriers before any can set it again
  ok = M > 0 && atomicOr(L.err, 0) == 0;
  if (timer) { const unsigned long long t = lw_now(); atomicAdd(&L.stats[LWS_SWEEP_FIRST_NS], t - t_mark); t_mark = t; }
  const bool sorted = ok && nlev <= kLwLevels;
  if (sorted) {
    // 2. counting sort by level (levels are 1 .. nlev); each position's row
    //    is copied to its sorted slot
    for (int p = t0; p < M; p += T) atomicAdd(&hist[*cluster.map_shared_rank(lvl + (p >> lc), p & (C - 1)) - 1], 1);
    cluster.sync();
    const int per = (nlev + (int)blockDim.x - 1) / (int)blockDim.x;
    const int l0 = min(nlev, (int)threadIdx.x * per), l1 = min(nlev, l0 + per);
    int sum = 0;
    for (int l = l0; l < l1; ++l) {
      int tot = 0, mine = 0;
      for (int c = 0; c < C; ++c) {
        const int v = *cluster.map_shared_rank(&hist[l], c);
        tot += v;
        if (c < rank) mine += v;
      }
      base[l] = mine;
      ltot[l] = tot;
      sum += tot;
    }
    const int wl = (int)threadIdx.x & 31, ww = (int)threadIdx.x >> 5;
    const int incl = warp_incl_scan(sum, wl);
    if (wl == 31) wsum[ww] = incl;
    __syncthreads();
    if (ww == 0) {
      const int v = (wl < ((int)blockDim.x >> 5)) ? wsum[wl] : 0;
      wsum[wl] = warp_incl_scan(v, wl);
    }
    __syncthreads();
    int run = (ww > 0 ? wsum[ww - 1] : 0) + incl - sum;
    for (int l = l0; l < l1; ++l) {
      const int t = ltot[l];
      ltot[l] = run;
      base[l] += run;
      run += t;
    }
    if (threadIdx.x == 0) ltot[nlev] = M;
    cluster.sync();
    for (int p = t0; p < M; p += T) {
      const int slot = atomicAdd(&base[*cluster.map_shared_rank(lvl + (p >> lc), p & (C - 1)) - 1], 1);
      const int r = L.prec[p].x;
      float4 rw[8];
      load_row(rows, r, rw);
      rw[7].w = __int_as_float(r);
      float4* dst = reinterpret_cast<float4*>(L.rsort + (size_t)slot * kRowWords);
#pragma unroll
      for (int q = 0; q < 8; ++q) dst[q] = rw[q];
    }
    cluster.sync();
    if (timer) {
      const unsigned long long t = lw_now();
      atomicAdd(&L.stats[LWS_SWEEP_SORT_NS], t - t_mark);
      t_mark = t;
    }
    // 3. level by level; slot a + k of a level goes to CTA k & (C-1), so every
    //    level is spread over the whole cluster
    const int tl = ((int)threadIdx.x << lc) + rank;
    for (int it = it0; it < it1; ++it) {
      LwRow R;
      bool have = false;
      {
        const int j = ltot[0] + tl;
        if (j < ltot[1]) { lw_load_sorted(L, j, R); have = true; }
      }
      for (int l = 0; l < nlev; ++l) {
        if (have) {
          lw_update(cluster, C, bodies, lam, R, 0u, L, nullptr, false);
          for (int j = ltot[l] + tl + T; j < ltot[l + 1]; j += T) {
            LwRow Rx;
            lw_load_sorted(L, j, Rx);
            lw_update(cluster, C, bodies, lam, Rx, 0u, L, nullptr, false);
          }
        }
        lw_arrive();
        // the next level's first row of this thread loads during the barrier
        have = false;
        if (l + 1 < nlev) {
          const int j = ltot[l + 1] + tl;
          if (j < ltot[l + 2]) { lw_load_sorted(L, j, R); have = true; }
        }
        lw_wait_all();
      }
    }
  } else if (ok) {
    // order position as bounded dataflow (levels deeper than the histogram)
    bool run_ok = true;
    for (int it = it0; run_ok && it < it1; ++it) {
      const unsigned li = (unsigned)(it - it0);
      LwRow cur, nxt;
      if (t0 < M) lw_load(rows, L, t0, cur);
      for (int j = t0; run_ok && j < M; j += T) {
        if (j + T < M) lw_load(rows, L, j + T, nxt);
        if (!lw_update(cluster, C, bodies, lam, cur, li, L, nullptr)) { run_ok = false; break; }
        cur = nxt;
      }
    }
  }
  cluster.sync();
  if (timer) {
    atomicAdd(&L.stats[LWS_SWEEP_REST_NS], lw_now() - t_mark);
    atomicMax(&L.stats[LWS_LEVELS_MAX], (unsigned long long)nlev);
    atomicAdd(&L.stats[LWS_SWEEPS], 1ull);
    L.stats[LWS_CLUSTER] = (unsigned long long)C;
  }
  for (int s = threadIdx.x; s < nbs; s += blockDim.x) {
    const int b = (s << lc) + rank;
    if (b < nb)
      for (int k = 0; k < 6; ++k) L.fc[6 * (size_t)b + k] = bodies[s].f[k];
  }
  for (int s = threadIdx.x; s < nrs; s += blockDim.x) {
    const int r = (s << lc) + rank;
    if (r < M) L.lambda[r] = lam[s];
  }
}

// ---------------------------------------------------------------- integration
// Joint feedback (quickstep.cpp:918-957, Multiply1_12q1 :70-101), a thread per
// island-ordered joint: f1 t1 = J1^T lambda and f2 t2 = J2^T lambda over the
// joint's rows in order, J as getInfo2 produced it (jcopy); f2 = t2 = 0
// without a second body. Persistent joints into feedback[joint][12], contact
// joints into contact_feedback[contact][12] (either may be null).
__global__ void lw_feedback_kernel(BatchDev d, LWDev L, const float* jcopy, float* feedback,
                                   float* contact_feedback) {
  const WorldDesc D = d.world[0];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (d.nrows[0] == 0 || k >= *L.nj) return;
  const int ord = L.jlist[k];
  float* o;
  int b2;
  if (ord < D.njp) {
    if (!feedback) return;
    o = feedback + (size_t)(D.joint_off + ord) * 12;
    b2 = d.joints[D.joint_off + ord].b2;
  } else {
    if (!contact_feedback) return;
    o = contact_feedback + (size_t)(D.contact_off + ord - D.njp) * 12;
    b2 = d.contacts[D.contact_off + ord - D.njp].b2;
  }
  float f[12];
  for (int q = 0; q < 12; ++q) f[q] = 0.f;
  for (int r = L.jm[k]; r < L.jm[k + 1]; ++r) {
    const float s = L.lambda[r];
    const float* J = jcopy + (size_t)(D.row_off + r) * 12;
    for (int q = 0; q < 12; ++q) f[q] += J[q] * s;
  }
  if (b2 < 0)
    for (int q = 6; q < 12; ++q) f[q] = 0.f;
  for (int q = 0; q < 12; ++q) o[q] = f[q];
}

__global__ void lw_integrate_kernel(BatchDev d, LWDev L) {
  const WorldDesc D = d.world[0];
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int M = d.nrows[0];
  if (b == 0) {
    const unsigned total = (unsigned)L.draws[d.nislands[0]];
    const unsigned seed = d.seed[0];
    if (M > 0) d.seed[0] = lcg_jump(seed, total);
    if (*L.err) atomicOr(&d.status[0], ST_SOLVE_STALL);
  }
  if (b >= L.nb) return;
  const bool bad = integrate_body(d, D, D.body_off + b, M > 0 ? L.fc + 6 * (size_t)b : nullptr);
  if (bad) atomicOr(&d.status[0], ST_NONFINITE);
}

}  // namespace og
