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
#include "joints.cuh"

namespace og {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxB = 64;      // bodies per world handled on chip
constexpr int kMaxR = 1024;    // constraint rows per world handled on chip

// Per-warp shared-memory working set of the setup phases.
struct WarpSmem {
  float* fc;          // [kMaxB*6]  tmp1 = invM fe + v/h per body
  int* cnt;           // [kMaxB+1]  contacts per body
  int16_t* stack;     // [kMaxB]    island search stack
  uint8_t* tag;       // [kMaxB]    body tags for the island search
  uint8_t* jtag;      // [kMaxR]    joint tags for the island search
};
constexpr int kSmemPerWarp = kMaxB * 6 * 4 + (kMaxB + 1) * 4 + kMaxB * 2 + kMaxB + kMaxR + 12;

OG_D WarpSmem carve_smem(unsigned char* base) {
  WarpSmem s;
  unsigned char* p = base;
  s.fc = reinterpret_cast<float*>(p); p += kMaxB * 6 * 4;
  s.cnt = reinterpret_cast<int*>(p); p += (kMaxB + 1) * 4;
  s.stack = reinterpret_cast<int16_t*>(p); p += kMaxB * 2;
  s.tag = p; p += kMaxB;
  s.jtag = p; p += kMaxR;
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

// Phase 1: canonical pair loop. Returns the number of contacts stored.
OG_D int phase_collide(const BatchDev& d, const WorldDesc& D, int w, int lane) {
  const int ng = D.ng;
  const int npairs = ng * (ng - 1) / 2;
  int nc = 0;
  for (int base = 0; base < npairs; base += 32) {
    const int p = base + lane;
    int cnt = 0;
    Contact cc[8];
    int bi = -1, bk = -1, surf = 0;
    if (p < npairs) {
      // unrank p -> (i, k), i < k, row-major over i
      const float tn = 2.f * ng - 1.f;
      int i = (int)floorf((tn - sqrtf(fmaxf(tn * tn - 8.f * p, 0.f))) * 0.5f);
      i = max(0, min(i, ng - 2));
      while (i > 0 && i * (2 * ng - i - 1) / 2 > p) --i;
      while ((i + 1) * (2 * ng - (i + 1) - 1) / 2 <= p) ++i;
      const int k = p - i * (2 * ng - i - 1) / 2 + i + 1;
      const int gi = D.geom_off + i, gk = D.geom_off + k;
      bi = d.gbody[gi];
      bk = d.gbody[gk];
      bool skip = (bi < 0 && bk < 0) || (bi == bk);
      if (!skip && bi >= 0 && bk >= 0 && jointed(d, D, w, bi, bk)) skip = true;
      if (!skip) {
        const float ri = d.gbound[gi], rk = d.gbound[gk];
        if (isfinite(ri) && isfinite(rk)) {
          const float4 pi4 = d.pos[D.body_off + bi], pk4 = d.pos[D.body_off + bk];
          const float dx = pi4.x - pk4.x, dy = pi4.y - pk4.y, dz = pi4.z - pk4.z;
          const float lim = (ri + rk) * 1.001f + 1e-5f;
          if (dx * dx + dy * dy + dz * dz > lim * lim) skip = true;
        }
      }
      if (!skip) {
        GeomView vi, vk;
        geom_view(d, D, i, vi);
        geom_view(d, D, k, vk);
        cnt = collide_primitive(vi, vk, (unsigned)D.max_contacts, cc);
        const int si = d.gsurf[gi], sk = d.gsurf[gk];
        surf = si > sk ? si : sk;
      }
    }
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
        ct.pad = 0;
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

// Phase 3: adjacency in ODE list order + DFS islands. Writes jlist (joint
// ordinals in island order; bit 30 marks the first joint of an island) and
// returns the number of joints placed; *n_isl receives the island count.
// nc_lists: contacts to merge into the body lists (0 when the host supplied
// complete lists in padj); nj_all: persistent + contact joints (tag range).
OG_D int phase_islands(const BatchDev& d, const WorldDesc& D, int w, int nc, int nj_all,
                       const WarpSmem& S, int lane, int* n_isl) {
  const int nb = D.nb;
  const int jl_off = D.joint_off + D.contact_off;
  const int adj_off = 2 * jl_off;
  int* adj_start = d.adj_start + D.body_off + w;
  // counts: contacts per body + persistent joints per body
  for (int b = lane; b < nb; b += 32) S.cnt[b] = 0;
  __syncwarp();
  for (int c = lane; c < nc; c += 32) {
    const DevContact& ct = d.contacts[D.contact_off + c];
    atomicAdd(&S.cnt[ct.b1], 1);
    if (ct.b2 >= 0) atomicAdd(&S.cnt[ct.b2], 1);
  }
  __syncwarp();
  const int* pstart = d.padj_start + D.body_off + w;
  {
    int carry = 0;
    for (int base = 0; base < nb; base += 32) {
      const int b = base + lane;
      const int v = (b < nb) ? S.cnt[b] + (pstart[b + 1] - pstart[b]) : 0;
      const int incl = warp_incl_scan(v, lane);
      if (b < nb) adj_start[b] = carry + incl - v;
      carry += __shfl_sync(kFull, incl, 31);
    }
    if (lane == 0) adj_start[nb] = carry;
  }
  __syncwarp();
  // fill: contacts newest first, then persistent joints newest first
  for (int b = lane; b < nb; b += 32) {
    int wp = adj_off + adj_start[b];
    for (int c = nc - 1; c >= 0; --c) {
      const DevContact& ct = d.contacts[D.contact_off + c];
      if (ct.b1 == b || ct.b2 == b) d.adj[wp++] = D.njp + c;
    }
    for (int k = pstart[b]; k < pstart[b + 1]; ++k) d.adj[wp++] = d.padj[k];
  }
  const int nj = nj_all;
  for (int b = lane; b < nb; b += 32) S.tag[b] = 0;
  for (int j = lane; j < nj; j += 32) S.jtag[j] = 0;
  __syncwarp();
  int jcount = 0, nisl = 0;
  if (lane == 0) {
    for (int bb = nb - 1; bb >= 0; --bb) {
      if (S.tag[bb]) continue;
      S.tag[bb] = 1;
      const int jstart = jcount;
      int sp = 0, b = bb;
      for (;;) {
        const int e = adj_start[b + 1];
        for (int k = adj_start[b]; k < e; ++k) {
          const int j = d.adj[adj_off + k];
          if (S.jtag[j]) continue;
          S.jtag[j] = 1;
          d.jlist[jl_off + jcount] = j | (jcount == jstart ? (1 << 30) : 0);
          ++jcount;
          int b1, b2;
          joint_bodies(d, D, j, b1, b2);
          const int other = (b1 == b) ? b2 : b1;
          if (other >= 0 && !S.tag[other]) {
            S.tag[other] = 1;
            S.stack[sp++] = (int16_t)other;
          }
        }
        if (sp == 0) break;
        b = S.stack[--sp];
      }
      if (jcount > jstart) {
        d.island_jstart[D.body_off + w + nisl] = jstart;
        ++nisl;
      }
    }
    d.island_jstart[D.body_off + w + nisl] = jcount;
  }
  jcount = __shfl_sync(kFull, jcount, 0);
  nisl = __shfl_sync(kFull, nisl, 0);
  __syncwarp();
  *n_isl = nisl;
  return jcount;
}

}  // namespace og
