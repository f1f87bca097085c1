// world_step.cuh -- one ODE world step executed by ONE warp.
//
// Phases (each cites the reference code it replaces):
//   0  controls into force/torque accumulators (dJointAddHingeTorque,
//      dJointAddHinge2Torques, dBodyAddForce/Torque)
//   1  narrowphase over the canonical pair order (dCollide, collision_kernel.cpp:292)
//   2  body prologue: world inverse inertia, gyroscopic torque, gravity
//      (dxQuickStepper, quickstep.cpp:600-665)
//   3  islands in ODE's DFS order (util.cpp:384-521)
//   4  getInfo1 / getInfo2 row assembly with findex rebasing (quickstep.cpp:670-830)
//   5  rhs, cfm/h, invM*J^T, Ad, J/b scaling (quickstep.cpp:832-857, :117-136, :370-402)
//   6  SOR_LCP sweeps with ODE's row order and seeded shuffle (quickstep.cpp:405-583)
//   7  velocity update + dxStepBody integration (quickstep.cpp:905-1021, util.cpp:255-360)
//
// The SOR phase is a "wavefront" Gauss-Seidel: each window of 32 consecutive
// rows (in the current sweep order) is split into dependency levels so that two
// rows of one level never touch the same body; levels run one after another.
// Every body therefore sees exactly the same sequence of updates as in ODE's
// sequential loop, and friction rows read lambda[findex] at the same point of
// that sequence (a friction row and its normal row share their bodies).
#pragma once
#include "collide.cuh"
#include "heightfield.cuh"
#include "joints.cuh"

namespace og {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxB = 64;      // bodies per world handled on chip
constexpr int kMaxR = 1024;    // constraint rows per world handled on chip

// Per-warp shared-memory working sets of the collide and build kernels.
struct WarpSmem {
  // build kernel
  float* fc;          // [kMaxB*6]   tmp1 = invM fe + v/h per body
  int* cnt;           // [kMaxB+1]   contacts per body, then list cursors
  uint16_t* adj_start;// [kMaxB+1]   body joint lists (CSR)
  uint16_t* adj;      // [2*kMaxR]   joint ordinals, ODE list order
  int8_t* jb1;        // [kMaxR]     bodies of each joint ordinal
  int8_t* jb2;        // [kMaxR]
  uint16_t* jlist;    // [kMaxR]     joints in island order (bit 15: island start)
  int16_t* stack;     // [kMaxB]     island search stack
  uint8_t* tag;       // [kMaxB]     body tags for the island search
  uint8_t* jtag;      // [kMaxR]     joint tags for the island search
  // collide kernel
  uint16_t* cand;     // [kMaxPairs] candidate pairs that pass the bound test
  float4* gpb;        // [kMaxB+8]   per geom: position (its body's, or its own when static), bound radius
  int16_t* gbd;       // [kMaxB+8]   per geom: body, -1 static
  unsigned long long* jmask;   // [kMaxB] per body: the bodies a persistent joint joins it to
};
constexpr int kMaxPairs = (kMaxB + 8) * (kMaxB + 7) / 2;   // geoms: bodies + a few static
// Per-warp sizes are rounded up to 16 bytes so that every warp's slice (and
// the float/int arrays at its start) stays aligned.
constexpr int align16(int n) { return (n + 15) & ~15; }
constexpr int kSmemPerWarp = align16(kMaxB * 6 * 4 + (kMaxB + 1) * 4 + (kMaxB + 1) * 2 + 2 * kMaxR * 2 +
                                     kMaxR * 2 + kMaxR * 2 + kMaxB * 2 + kMaxB + kMaxR + 32);
constexpr int kCollideSmemPerWarp = align16(kMaxPairs * 2 + 16) + align16((kMaxB + 8) * 16) + align16((kMaxB + 8) * 2) +
                                    align16(kMaxB * 8);
static_assert(kSmemPerWarp % 16 == 0 && kCollideSmemPerWarp % 16 == 0, "per-warp slices must stay aligned");
static_assert(kMaxB * 6 * sizeof(float) >= 6 * kMaxB * sizeof(int), "the island phase borrows the tmp1 area");

OG_D WarpSmem carve_smem(unsigned char* base) {
  WarpSmem s;
  unsigned char* p = base;
  s.fc = reinterpret_cast<float*>(p); p += kMaxB * 6 * 4;
  s.cnt = reinterpret_cast<int*>(p); p += (kMaxB + 1) * 4;
  s.adj = reinterpret_cast<uint16_t*>(p); p += 2 * kMaxR * 2;
  s.jlist = reinterpret_cast<uint16_t*>(p); p += kMaxR * 2;
  s.adj_start = reinterpret_cast<uint16_t*>(p); p += (kMaxB + 1) * 2 + 2;
  s.stack = reinterpret_cast<int16_t*>(p); p += kMaxB * 2;
  s.jb1 = reinterpret_cast<int8_t*>(p); p += kMaxR;
  s.jb2 = reinterpret_cast<int8_t*>(p); p += kMaxR;
  s.tag = p; p += kMaxB;
  s.jtag = p; p += kMaxR;
  s.cand = nullptr;
  return s;
}
OG_D WarpSmem carve_collide_smem(unsigned char* base) {
  WarpSmem s{};
  s.cand = reinterpret_cast<uint16_t*>(base);
  base += align16(kMaxPairs * 2 + 16);
  s.gpb = reinterpret_cast<float4*>(base);
  base += align16((kMaxB + 8) * 16);
  s.gbd = reinterpret_cast<int16_t*>(base);
  base += align16((kMaxB + 8) * 2);
  s.jmask = reinterpret_cast<unsigned long long*>(base);
  return s;
}

OG_D int warp_incl_scan(int v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += t;
  }
  return v;
}
OG_D int warp_max(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// Rotation of a body from its quaternion (the reference keeps R in sync with q
// through dRfromQ after every change, so recomputing it is equivalent).
OG_D void body_R(const BatchDev& d, int gb, float* R) {
  const float4 q = d.q[gb];
  const float qq[4] = {q.x, q.y, q.z, q.w};
  r_from_q(R, qq);
}

OG_D void geom_view(const BatchDev& d, const WorldDesc& D, int g, GeomView& v) {
  const int gg = D.geom_off + g;
  v.type = d.gtype[gg];
  const float4 p = d.gparam[gg];
  v.p[0] = p.x; v.p[1] = p.y; v.p[2] = p.z; v.p[3] = p.w;
  const int b = d.gbody[gg];
  if (b >= 0) {
    const float4 ps = d.pos[D.body_off + b];
    v.pos[0] = ps.x; v.pos[1] = ps.y; v.pos[2] = ps.z;
    body_R(d, D.body_off + b, v.R);
  } else {
    const float4 ps = d.gpos[gg];
    v.pos[0] = ps.x; v.pos[1] = ps.y; v.pos[2] = ps.z;
    for (int k = 0; k < 12; ++k) v.R[k] = 0.f;
    v.R[0] = v.R[5] = v.R[10] = 1.f;
  }
}

// Are bodies b1 and b2 joined by a persistent joint? (the near-callback's
// dAreConnectedExcluding(b1, b2, dJointTypeContact), ode/src/ode.cpp:1529-1537)
OG_D bool jointed(const BatchDev& d, const WorldDesc& D, int w, int b1, int b2) {
  const int s = d.padj_start[D.body_off + w + b1], e = d.padj_start[D.body_off + w + b1 + 1];
  for (int k = s; k < e; ++k) {
    const DevJoint& J = d.joints[D.joint_off + d.padj[k]];
    const int other = (J.b1 == b1) ? J.b2 : J.b1;
    if (other == b2) return true;
  }
  return false;
}

OG_D void unrank_pair(int p, int ng, int& i, int& k) {
  // p -> (i, k), i < k, row-major over i
  const float tn = 2.f * ng - 1.f;
  i = (int)floorf((tn - sqrtf(fmaxf(tn * tn - 8.f * p, 0.f))) * 0.5f);
  i = max(0, min(i, ng - 2));
  while (i > 0 && i * (2 * ng - i - 1) / 2 > p) --i;
  while ((i + 1) * (2 * ng - (i + 1) - 1) / 2 <= p) ++i;
  k = p - i * (2 * ng - i - 1) / 2 + i + 1;
}

// dCollide(g_i, g_k) for a pair with a heightfield: the heightfield collider
// runs with the field first and the normals are negated when the call was
// reversed (collision_kernel.cpp:320-334). Returns the contact count, 0 for
// geoms the heightfield has no collider for, or -1 when the zone under the
// geom exceeds the lane's arrays and the workspace `big`.
OG_D int collide_hf_pair(const BatchDev& d, const GeomView& vi, const GeomView& vk, unsigned flags, Contact* cc,
                         unsigned* kinds, HFBig big) {
  const bool rev = vk.type == G_HEIGHTFIELD;
  const GeomView& hv = rev ? vk : vi;
  const GeomView& ov = rev ? vi : vk;
  if (!(ov.type == G_SPHERE || ov.type == G_BOX || ov.type == G_CAPSULE || ov.type == G_CYLINDER)) return 0;
  const int cnt = collide_heightfield(d.hfs[(int)hv.p[0]], d.hf_heights, ov, flags, cc, kinds, big);
  if (rev)
    for (int c = 0; c < cnt; ++c) {
      cc[c].normal[0] = -cc[c].normal[0]; cc[c].normal[1] = -cc[c].normal[1];
      cc[c].normal[2] = -cc[c].normal[2];
    }
  return cnt;
}

// Phase 1: canonical pair loop. A first pass keeps, in pair order, the pairs
// that the dCollide early-outs and a conservative bounding-sphere test cannot
// reject; the colliders then run densely over those candidates and a warp
// prefix scan writes the contacts in pair order. Returns the contact count.
OG_D int phase_collide(const BatchDev& d, const WorldDesc& D, int w, const WarpSmem& S, int lane) {
  const int ng = D.ng;
  const int npairs = ng * (ng - 1) / 2;
  // the world's geoms for the candidate pass, staged once: body, position
  // (a static geom's own) and bounding radius
  for (int g = lane; g < ng; g += 32) {
    const int gg = D.geom_off + g;
    const int b = d.gbody[gg];
    const float4 p = b >= 0 ? d.pos[D.body_off + b] : d.gpos[gg];
    S.gpb[g] = make_float4(p.x, p.y, p.z, d.gbound[gg]);
    S.gbd[g] = (int16_t)b;
  }
  // the pairs of bodies a persistent joint joins, as one bit mask per body:
  // the near-callback's dAreConnectedExcluding(b1, b2, dJointTypeContact)
  // test (ode/src/ode.cpp:1529-1537) becomes one shared-memory load
  for (int b = lane; b < D.nb; b += 32) S.jmask[b] = 0ull;
  __syncwarp();
  for (int j = lane; j < D.njp; j += 32) {
    const DevJoint& J = d.joints[D.joint_off + j];
    if (J.b1 >= 0 && J.b2 >= 0) {
      atomicOr(&S.jmask[J.b1], 1ull << J.b2);
      atomicOr(&S.jmask[J.b2], 1ull << J.b1);
    }
  }
  __syncwarp();
  int ncand = 0;
  // this lane's pair (i, k) of the canonical order, advanced 32 pairs a round
  int pi = 0, pk = 1;
  if (lane < npairs) unrank_pair(lane, ng, pi, pk);
  for (int base = 0; base < npairs; base += 32) {
    const int p = base + lane;
    bool keep = false;
    if (p < npairs) {
      const int i = pi, k = pk;
      const int bi = S.gbd[i], bk = S.gbd[k];
      keep = !((bi < 0 && bk < 0) || (bi == bk));
      if (keep) {
        const float4 pi4 = S.gpb[i], pk4 = S.gpb[k];
        if (isfinite(pi4.w) && isfinite(pk4.w)) {
          const float dx = pi4.x - pk4.x, dy = pi4.y - pk4.y, dz = pi4.z - pk4.z;
          const float lim = (pi4.w + pk4.w) * 1.001f + 1e-5f;
          if (dx * dx + dy * dy + dz * dz > lim * lim) keep = false;
        }
      }
      if (keep && bi >= 0 && bk >= 0 && ((S.jmask[bi] >> bk) & 1ull)) keep = false;
      // 32 pairs on: row i holds the pairs (i, i+1 .. ng-1)
      pk += 32;
      while (pk >= ng && pi < ng - 2) {
        const int over = pk - ng;
        ++pi;
        pk = pi + 1 + over;
      }
    }
    const unsigned bal = __ballot_sync(kFull, keep);
    if (keep) S.cand[ncand + __popc(bal & ((1u << lane) - 1u))] = (uint16_t)p;
    ncand += __popc(bal);
  }
  __syncwarp();
  int nc = 0;
  for (int base = 0; base < ncand; base += 32) {
    const int ci = base + lane;
    int cnt = 0;
    Contact cc[8];
    int bi = -1, bk = -1, surf = 0, pair = -1;
    unsigned kinds = 0u;
    if (ci < ncand) {
      int i, k;
      unrank_pair(S.cand[ci], ng, i, k);
      pair = i | (k << 8);
      const int gi = D.geom_off + i, gk = D.geom_off + k;
      bi = d.gbody[gi];
      bk = d.gbody[gk];
      GeomView vi, vk;
      geom_view(d, D, i, vi);
      geom_view(d, D, k, vk);
      if (vi.type == G_HEIGHTFIELD || vk.type == G_HEIGHTFIELD)
        cnt = collide_hf_pair(d, vi, vk, (unsigned)D.max_contacts, cc, &kinds, HFBig{nullptr, 0});
      else
        cnt = collide_primitive(vi, vk, (unsigned)D.max_contacts, cc);
      const int si = d.gsurf[gi], sk = d.gsurf[gk];
      surf = si > sk ? si : sk;
    }
    // heightfield zones beyond the lane's arrays: one lane at a time through
    // the world's workspace (worlds whose geoms can need one have it)
    if (D.hf_ws_side > 0) {
      unsigned big = __ballot_sync(kFull, cnt < 0);
      while (big) {
        const int l = __ffs(big) - 1;
        big &= big - 1;
        if (lane == l) {
          int i, k;
          unrank_pair(S.cand[ci], ng, i, k);
          GeomView vi, vk;
          geom_view(d, D, i, vi);
          geom_view(d, D, k, vk);
          cnt = collide_hf_pair(d, vi, vk, (unsigned)D.max_contacts, cc, &kinds,
                                HFBig{d.hf_ws + D.hf_ws, D.hf_ws_side});
        }
        __syncwarp();
      }
    }
    if (cnt < 0) { atomicOr(&d.status[w], ST_HF_ZONE); cnt = 0; }
    const int incl = warp_incl_scan(cnt, lane);
    const int excl = incl - cnt;
    const int total = __shfl_sync(kFull, incl, 31);
    for (int c = 0; c < cnt; ++c) {
      const int slot = nc + excl + c;
      if (slot < D.contact_cap) {
        DevContact ct;
        ct.pos[0] = cc[c].pos[0]; ct.pos[1] = cc[c].pos[1]; ct.pos[2] = cc[c].pos[2];
        ct.depth = cc[c].depth;
        ct.normal[0] = cc[c].normal[0]; ct.normal[1] = cc[c].normal[1]; ct.normal[2] = cc[c].normal[2];
        ct.surface = surf;
        // dJointAttach(body(gi), body(gk)): a missing first body swaps in the second
        if (bi < 0) { ct.b1 = bk; ct.b2 = -1; ct.reverse = 1; }
        else { ct.b1 = bi; ct.b2 = bk; ct.reverse = 0; }
        ct.geoms = pair | (int)(((kinds >> (2 * c)) & 3u) << 16);
        d.contacts[D.contact_off + slot] = ct;
      }
    }
    nc += total;
  }
  if (nc > D.contact_cap) {
    if (lane == 0) atomicOr(&d.status[w], ST_CONTACT_OVERFLOW);
    nc = D.contact_cap;
  }
  return nc;
}

OG_D void joint_bodies(const BatchDev& d, const WorldDesc& D, int ord, int& b1, int& b2) {
  if (ord < D.njp) {
    const DevJoint& J = d.joints[D.joint_off + ord];
    b1 = J.b1; b2 = J.b2;
  } else {
    const DevContact& c = d.contacts[D.contact_off + ord - D.njp];
    b1 = c.b1; b2 = c.b2;
  }
}

// Phase 3: adjacency in ODE list order + islands in ODE's DFS order
// (util.cpp:384-521), all in shared memory. Body lists hold contacts newest
// first, then persistent joints newest first (nc = 0 when the host supplied
// complete lists in padj). Writes jlist (joint ordinals in island order; bit
// 15 marks an island's first joint) and island_jstart; returns the number of
// joints placed.
//
// The reference walks the bodies from the last one down and runs a
// depth-first search from every body not yet reached; the body that starts an
// island is therefore the largest of its connected component, islands come in
// decreasing order of that body, and an island's joints come in the order its
// search first meets them. Here the components are labelled first, lanes in
// parallel (every body takes the largest label among its neighbours, with
// pointer jumping, until nothing changes), which gives every island's start
// body, joint count and place in jlist; then each island's search runs on a
// lane of its own, in the reference's order, with a slice of the stack sized
// by its body count. Islands are disjoint, so the lanes never touch the same
// body or joint.
OG_D int phase_islands(const BatchDev& d, const WorldDesc& D, int w, int nc, int nj_all,
                       const WarpSmem& S, int lane, int* n_isl) {
  const int nb = D.nb;
  const int* pstart = d.padj_start + D.body_off + w;
  const unsigned below = (1u << lane) - 1u;
  // per-body scratch in the (not yet used) tmp1 area: 6 x kMaxB ints
  int* lab = reinterpret_cast<int*>(S.fc);   // component label: its largest body
  int* jcnt = lab + kMaxB;                   // joints of the component (by label)
  int* bcnt = jcnt + kMaxB;                  // bodies of the component (by label)
  int* jst = bcnt + kMaxB;                   // first jlist slot of the island (by start body)
  int* sst = jst + kMaxB;                    // first stack slot of the island (by start body)
  int* iroot = sst + kMaxB;                  // start body of island i, in island order
  // bodies of every joint ordinal
  for (int j = lane; j < nj_all; j += 32) {
    int b1, b2;
    joint_bodies(d, D, j, b1, b2);
    S.jb1[j] = (int8_t)b1;
    S.jb2[j] = (int8_t)b2;
    S.jtag[j] = 0;
  }
  for (int b = lane; b < nb; b += 32) {
    S.cnt[b] = 0; S.tag[b] = 0; S.stack[b] = 0;
    lab[b] = b; jcnt[b] = 0; bcnt[b] = 0;
  }
  __syncwarp();
  for (int c = lane; c < nc; c += 32) {
    atomicAdd(&S.cnt[S.jb1[D.njp + c]], 1);
    if (S.jb2[D.njp + c] >= 0) atomicAdd(&S.cnt[S.jb2[D.njp + c]], 1);
  }
  __syncwarp();
  {
    int carry = 0;
    for (int base = 0; base < nb; base += 32) {
      const int b = base + lane;
      const int v = (b < nb) ? S.cnt[b] + (pstart[b + 1] - pstart[b]) : 0;
      const int incl = warp_incl_scan(v, lane);
      if (b < nb) S.adj_start[b] = (uint16_t)(carry + incl - v);
      carry += __shfl_sync(kFull, incl, 31);
    }
    if (lane == 0) S.adj_start[nb] = (uint16_t)carry;
  }
  __syncwarp();
  // fill, contacts newest first: sixteen contacts per window, a contact's two
  // bodies on two lanes; an entry's place in its body's list is the body's
  // cursor (S.stack) plus the number of earlier entries in the window on the
  // same body (__match_any_sync)
  for (int base = 0; base < nc; base += 16) {
    const int ci = base + (lane >> 1);
    const int c = nc - 1 - ci;
    int body = -1;
    if (ci < nc) body = (lane & 1) ? S.jb2[D.njp + c] : S.jb1[D.njp + c];
    const bool valid = body >= 0;
    const unsigned mask = __match_any_sync(kFull, valid ? body : -1 - lane);
    const int rank = __popc(mask & below);
    if (valid) S.adj[S.adj_start[body] + S.stack[body] + rank] = (uint16_t)(D.njp + c);
    __syncwarp();
    if (valid && (mask >> lane) == 1u) S.stack[body] = (int16_t)(S.stack[body] + rank + 1);
    __syncwarp();
  }
  // then each body's persistent joints
  for (int b = lane; b < nb; b += 32) {
    int wp = S.adj_start[b] + S.cnt[b];
    for (int k = pstart[b]; k < pstart[b + 1]; ++k) S.adj[wp++] = (uint16_t)d.padj[k];
  }
  // components: largest label along every joint, pointer jumping, until stable
  for (;;) {
    bool changed = false;
    for (int j = lane; j < nj_all; j += 32) {
      const int b1 = S.jb1[j], b2 = S.jb2[j];
      if (b1 < 0 || b2 < 0) continue;
      const int l1 = lab[b1], l2 = lab[b2];
      if (l1 != l2) {
        const int m = max(l1, l2);
        atomicMax(&lab[b1], m);
        atomicMax(&lab[b2], m);
        changed = true;
      }
    }
    __syncwarp();
    for (int b = lane; b < nb; b += 32) {
      const int l = lab[b];
      const int ll = lab[l];
      if (ll > l) atomicMax(&lab[b], ll);
    }
    __syncwarp();
    if (!__any_sync(kFull, changed)) break;
  }
  // a component's island starts at its newest body that was enabled when the
  // step began (S.cnt is free again: by label, -1 for none)
  int* rt = S.cnt;
  for (int b = lane; b < nb; b += 32) rt[b] = -1;
  __syncwarp();
  for (int b = lane; b < nb; b += 32) {
    atomicAdd(&bcnt[lab[b]], 1);
    if (!(d.bflags[D.body_off + b] & BODY_WOKEN)) atomicMax(&rt[lab[b]], b);
  }
  for (int j = lane; j < nj_all; j += 32)
    if (S.jb1[j] >= 0) atomicAdd(&jcnt[lab[S.jb1[j]]], 1);
  __syncwarp();
  // islands: components with joints, by decreasing start body
  int jcount = 0, nisl = 0, scarry = 0;
  for (int base = 0; base < nb; base += 32) {
    const int b = nb - 1 - (base + lane);
    const int l = b >= 0 ? lab[b] : 0;
    const bool isl = b >= 0 && (rt[l] >= 0 ? rt[l] : l) == b && jcnt[l] > 0;
    const int jn = isl ? jcnt[l] : 0, bn = isl ? bcnt[l] : 0;
    const int ji = warp_incl_scan(jn, lane), bi = warp_incl_scan(bn, lane);
    const unsigned bal = __ballot_sync(kFull, isl);
    if (isl) {
      jst[b] = jcount + ji - jn;
      sst[b] = scarry + bi - bn;
      iroot[nisl + __popc(bal & below)] = b;
    }
    jcount += __shfl_sync(kFull, ji, 31);
    scarry += __shfl_sync(kFull, bi, 31);
    nisl += __popc(bal);
  }
  __syncwarp();
  // every island's depth-first search on a lane of its own
  int* istart = d.island_jstart + D.body_off + w;
  for (int i = lane; i < nisl; i += 32) {
    const int root = iroot[i];
    const int jstart = jst[root], sbase = sst[root];
    int jc = jstart, sp = 0, b = root;
    S.tag[root] = 1;
    for (;;) {
      const int e = S.adj_start[b + 1];
      for (int k = S.adj_start[b]; k < e; ++k) {
        const int j = S.adj[k];
        if (S.jtag[j]) continue;
        S.jtag[j] = 1;
        S.jlist[jc] = (uint16_t)(j | (jc == jstart ? 0x8000 : 0));
        ++jc;
        const int b1 = S.jb1[j], b2 = S.jb2[j];
        const int other = (b1 == b) ? b2 : b1;
        if (other >= 0 && !S.tag[other]) {
          S.tag[other] = 1;
          S.stack[sbase + sp++] = (int16_t)other;
        }
      }
      if (sp == 0) break;
      b = S.stack[sbase + --sp];
    }
    istart[i] = jstart;
  }
  if (lane == 0) istart[nisl] = jcount;
  // publish the joint order for the row phase
  const int jl_off = D.joint_off + D.contact_off;
  __syncwarp();
  for (int k = lane; k < jcount; k += 32) {
    const int v = S.jlist[k];
    d.jlist[jl_off + k] = (v & 0x7fff) | ((v & 0x8000) ? (1 << 30) : 0);
  }
  __syncwarp();
  *n_isl = nisl;
  return jcount;
}

}  // namespace og
