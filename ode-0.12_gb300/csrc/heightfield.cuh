// heightfield.cuh -- dCollideHeightfield (ode/src/heightfield.cpp:1677-1853)
// and dCollideHeightfieldZone (:952-1676) for sphere, box and capsule geoms,
// FP32 on the device (the reference's dSINGLE build: dEpsilon = FLT_EPSILON).
//
// One lane runs one (heightfield, geom) pair: the geom is moved into the
// heightfield's frame (Y up, origin at the field's centre), the sample zone
// under its AABB is gathered into lane-local arrays, the zone's triangles
// that reach above the geom's lowest point are grouped into planes (equal
// plane definitions within dEpsilon), the planes are sorted by height, each
// plane is collided with the geom's plane collider and every contact is kept
// if it lies over one of the plane's triangles (IsOnHeightfield2). Geoms
// larger than 1.5 cells then test the remaining triangle vertices with the
// geom's point-depth function. The edge pass is compiled out in the
// reference and here. Zones of up to kHFZone x kHFZone samples live in the
// lane's local memory; a larger zone needs a workspace in global memory from
// the caller (HFBig, up to kHFBigZone samples per axis), else it reports
// overflow and yields no contacts.
#pragma once
#include "collide.cuh"
#include "engine_types.cuh"

namespace og {

constexpr int kHFZone = 10;                                  // samples per axis
constexpr int kHFMaxTri = 2 * (kHFZone - 1) * (kHFZone - 1);
constexpr int kHFMaxcPerCell = 10;                           // HEIGHTFIELDMAXCONTACTPERCELL
constexpr float kHFEps = 1.1920928955078125e-07f;            // FLT_EPSILON
// How a heightfield contact arose (two bits per contact in `kinds`): the
// plane pass (a plane collider against a triangle's plane), the vertex pass
// (a field sample inside the geom), or the geom entirely under the field.
constexpr unsigned kHFPlane = 0u, kHFVertex = 1u, kHFUnder = 2u;

// GetHeight(int, int) (heightfield.cpp:302-364)
OG_D float hf_sample(const DevHeightfield& H, const float* heights, int x, int z) {
  if (H.wrap == 0) {
    x = x < 0 ? 0 : (x > H.nx - 1 ? H.nx - 1 : x);
    z = z < 0 ? 0 : (z > H.nz - 1 ? H.nz - 1 : z);
  } else {
    x %= H.nx - 1;
    z %= H.nz - 1;
    if (x < 0) x += H.nx - 1;
    if (z < 0) z += H.nz - 1;
  }
  return heights[H.h_off + x + z * H.nx] * H.scale + H.offset;
}

// IsOnHeightfield2 (heightfield.cpp:241-299); corner = A (up) or D (down)
OG_D bool hf_on_triangle(const DevHeightfield& H, const float* corner, int cx, int cz, const float* pos,
                         bool up) {
  if (up) {
    const float minx = corner[0];
    if (pos[0] < minx) return false;
    const float maxx = (cx + 1) * H.sw;
    if (pos[0] >= maxx) return false;
    const float minz = corner[2];
    if (pos[2] < minz) return false;
    const float maxz = (cz + 1) * H.sd;
    if (pos[2] >= maxz) return false;
    return (maxz - pos[2]) > (pos[0] - minx) * H.zx;
  }
  const float maxx = corner[0];
  if (pos[0] >= maxx) return false;
  const float minx = (cx - 1) * H.sw;
  if (pos[0] < minx) return false;
  const float maxz = corner[2];
  if (pos[2] >= maxz) return false;
  const float minz = (cz - 1) * H.sd;
  if (pos[2] < minz) return false;
  return (maxz - pos[2]) <= (pos[0] - minx) * H.zx;
}

// computeAABB of sphere / box / capsule / cylinder / ray (sphere.cpp:59-67,
// box.cpp:60-78, capsule.cpp:60-74, cylinder.cpp:58-73, ray.cpp:56-89)
OG_D void geom_aabb(const GeomView& g, float* aabb) {
  const float* R = g.R;
  float xr, yr, zr;
  if (g.type == G_RAY) {
    for (int i = 0; i < 3; ++i) {
      const float e = g.pos[i] + R[i * 4 + 2] * g.p[0];
      aabb[2 * i] = g.pos[i] < e ? g.pos[i] : e;
      aabb[2 * i + 1] = g.pos[i] < e ? e : g.pos[i];
    }
    return;
  }
  if (g.type == G_SPHERE) {
    xr = yr = zr = g.p[0];
  } else if (g.type == G_CYLINDER) {   // cylinder.cpp:58-73
    xr = fabsf(R[0] * g.p[0]) + fabsf(R[1] * g.p[0]) + 0.5f * fabsf(R[2] * g.p[1]);
    yr = fabsf(R[4] * g.p[0]) + fabsf(R[5] * g.p[0]) + 0.5f * fabsf(R[6] * g.p[1]);
    zr = fabsf(R[8] * g.p[0]) + fabsf(R[9] * g.p[0]) + 0.5f * fabsf(R[10] * g.p[1]);
  } else if (g.type == G_BOX) {
    xr = 0.5f * (fabsf(R[0] * g.p[0]) + fabsf(R[1] * g.p[1]) + fabsf(R[2] * g.p[2]));
    yr = 0.5f * (fabsf(R[4] * g.p[0]) + fabsf(R[5] * g.p[1]) + fabsf(R[6] * g.p[2]));
    zr = 0.5f * (fabsf(R[8] * g.p[0]) + fabsf(R[9] * g.p[1]) + fabsf(R[10] * g.p[2]));
  } else {
    xr = fabsf(R[2] * g.p[1]) * 0.5f + g.p[0];
    yr = fabsf(R[6] * g.p[1]) * 0.5f + g.p[0];
    zr = fabsf(R[10] * g.p[1]) * 0.5f + g.p[0];
  }
  aabb[0] = g.pos[0] - xr; aabb[1] = g.pos[0] + xr;
  aabb[2] = g.pos[1] - yr; aabb[3] = g.pos[1] + yr;
  aabb[4] = g.pos[2] - zr; aabb[5] = g.pos[2] + zr;
}

// dGeomSpherePointDepth (sphere.cpp:95-105), dGeomBoxPointDepth
// (box.cpp:109-172), dGeomCapsulePointDepth (capsule.cpp:104-126)
OG_D float geom_point_depth(const GeomView& g, const float* v) {
  const float* pos = g.pos;
  const float* R = g.R;
  if (g.type == G_SPHERE) {
    return g.p[0] - sqrtf((v[0] - pos[0]) * (v[0] - pos[0]) + (v[1] - pos[1]) * (v[1] - pos[1]) +
                          (v[2] - pos[2]) * (v[2] - pos[2]));
  }
  if (g.type == G_BOX) {
    const float p[3] = {v[0] - pos[0], v[1] - pos[1], v[2] - pos[2]};
    float q[3], dist[6];
    mul1_331(q, R, p);
    bool inside = true;
    for (int i = 0; i < 3; i++) {
      const float side = g.p[i] * 0.5f;
      dist[i] = side - q[i];
      dist[i + 3] = side + q[i];
      if ((dist[i] < 0.f) || (dist[i + 3] < 0.f)) inside = false;
    }
    if (inside) {
      float smallest = (float)(unsigned)-1;
      for (int i = 0; i < 6; i++)
        if (dist[i] < smallest) smallest = dist[i];
      return smallest;
    }
    float largest = 0.f;
    for (int i = 0; i < 6; i++)
      if (dist[i] > largest) largest = dist[i];
    return -largest;
  }
  float a[3] = {v[0] - pos[0], v[1] - pos[1], v[2] - pos[2]};
  float beta = a[0] * R[2] + a[1] * R[6] + a[2] * R[10];
  const float lz2 = g.p[1] * 0.5f;
  if (beta < -lz2) beta = -lz2;
  else if (beta > lz2) beta = lz2;
  a[0] = pos[0] + beta * R[2];
  a[1] = pos[1] + beta * R[6];
  a[2] = pos[2] + beta * R[10];
  return g.p[0] - sqrtf((v[0] - a[0]) * (v[0] - a[0]) + (v[1] - a[1]) * (v[1] - a[1]) +
                        (v[2] - a[2]) * (v[2] - a[2]));
}

OG_D int geom_plane_collide(const GeomView& g, const GeomView& pl, unsigned flags, Contact* c) {
  if (g.type == G_SPHERE) return collide_sphere_plane(g, pl, c);
  if (g.type == G_BOX) return collide_box_plane(g, pl, flags, c);
  if (g.type == G_RAY) return collide_ray_plane(g, pl, c);
  if (g.type == G_CYLINDER) return collide_cylinder_plane(g, pl, flags, c);
  return collide_capsule_plane(g, pl, flags, c);
}

// Working arrays of one zone (the reference's tempHeightBuffer,
// tempTriangleBuffer and tempPlaneBuffer, heightfield.cpp:1120-1140). A
// triangle's vertex indices are packed in a TV word, kTVBits bits each, with
// its "up" flag above them; Idx holds triangle and plane indices.
//   HFLocalZone: zones of up to kHFZone x kHFZone samples, in the lane's local
//     memory (every zone of the workloads' geoms);
//   HFGlobalZone: larger zones, up to kHFBigZone samples per axis, in a
//     workspace in global memory that the caller owns.
struct HFLocalZone {
  using TV = unsigned;
  using Idx = unsigned char;
  static constexpr int kTVBits = 8;
  float vh[kHFZone * kHFZone];           // sample heights of the zone
  unsigned char vstate[kHFZone * kHFZone];
  TV tv[kHFMaxTri];
  float4 tp[kHFMaxTri];                  // plane (n, d)
  float tmax[kHFMaxTri];                 // highest vertex
  unsigned char tstate[kHFMaxTri];
  Idx members[kHFMaxTri];                // triangles, grouped by plane
  Idx pfirst[kHFMaxTri], pcount[kHFMaxTri];
  float pmax[kHFMaxTri];
  Idx porder[kHFMaxTri];                 // planes in sorted order
  Idx tord[kHFMaxTri], trank[kHFMaxTri]; // triangles by plane offset, and each one's place there
};
constexpr int kHFBigZone = 128;          // samples per axis of a global workspace, at most
struct HFGlobalZone {
  using TV = unsigned long long;
  using Idx = unsigned short;
  static constexpr int kTVBits = 16;
  float* vh;
  unsigned char* vstate;
  TV* tv;
  float4* tp;
  float* tmax;
  unsigned char* tstate;
  Idx* members;
  Idx* pfirst;
  Idx* pcount;
  float* pmax;
  Idx* porder;
  Idx* tord;
  Idx* trank;
};
static_assert(kHFZone * kHFZone <= 256 && kHFMaxTri <= 255, "local zone indices are 8-bit");
static_assert(kHFBigZone * kHFBigZone <= 65536 && 2 * (kHFBigZone - 1) * (kHFBigZone - 1) <= 65535,
              "global zone indices are 16-bit");

// Bytes of a global workspace for zones of up to side x side samples.
OG_HD constexpr long long hf_ws_align(long long n) { return (n + 15) & ~15LL; }
OG_HD constexpr long long hf_ws_bytes(int side) {
  return hf_ws_align(4LL * side * side) + hf_ws_align(1LL * side * side) +
         hf_ws_align(8LL * 2 * (side - 1) * (side - 1)) + hf_ws_align(16LL * 2 * (side - 1) * (side - 1)) +
         hf_ws_align(4LL * 2 * (side - 1) * (side - 1)) + hf_ws_align(1LL * 2 * (side - 1) * (side - 1)) +
         3 * hf_ws_align(2LL * 2 * (side - 1) * (side - 1)) + hf_ws_align(4LL * 2 * (side - 1) * (side - 1)) +
         3 * hf_ws_align(2LL * 2 * (side - 1) * (side - 1));
}
OG_D HFGlobalZone carve_hf_ws(unsigned char* p, int side) {
  const long long S = (long long)side * side, T = 2LL * (side - 1) * (side - 1);
  HFGlobalZone z;
  z.vh = reinterpret_cast<float*>(p); p += hf_ws_align(4 * S);
  z.vstate = p; p += hf_ws_align(S);
  z.tv = reinterpret_cast<HFGlobalZone::TV*>(p); p += hf_ws_align(8 * T);
  z.tp = reinterpret_cast<float4*>(p); p += hf_ws_align(16 * T);
  z.tmax = reinterpret_cast<float*>(p); p += hf_ws_align(4 * T);
  z.tstate = p; p += hf_ws_align(T);
  z.members = reinterpret_cast<unsigned short*>(p); p += hf_ws_align(2 * T);
  z.pfirst = reinterpret_cast<unsigned short*>(p); p += hf_ws_align(2 * T);
  z.pcount = reinterpret_cast<unsigned short*>(p); p += hf_ws_align(2 * T);
  z.pmax = reinterpret_cast<float*>(p); p += hf_ws_align(4 * T);
  z.porder = reinterpret_cast<unsigned short*>(p); p += hf_ws_align(2 * T);
  z.tord = reinterpret_cast<unsigned short*>(p); p += hf_ws_align(2 * T);
  z.trank = reinterpret_cast<unsigned short*>(p);
  return z;
}

// A workspace for zones above kHFZone x kHFZone samples: ws (16-byte aligned,
// hf_ws_bytes(side) bytes) or null when the caller has none.
struct HFBig {
  unsigned char* ws;
  int side;
};

// dCollideHeightfieldZone (heightfield.cpp:952-1676); g in heightfield space,
// the zone's arrays in Z (which the caller has checked holds the zone).
// Returns the contact count.
template <class Z>
OG_D int hf_zone(Z& z, const DevHeightfield& H, const float* heights, int minX, int maxX, int minZ, int maxZ,
                 const GeomView& g, const float* aabb, int max_contacts, unsigned flags, Contact* out,
                 unsigned& kinds) {
  using TV = typename Z::TV;
  using Idx = typename Z::Idx;
  constexpr int kB = Z::kTVBits;
  constexpr TV kM = (TV(1) << kB) - 1;
  kinds = 0u;
  const int numX = (maxX - minX) + 1, numZ = (maxZ - minZ) + 1;
  const float minO2 = aabb[2], maxO2 = aabb[3];
  float* vh = z.vh;
  unsigned char* vstate = z.vstate;
  float maxY = -INFINITY, minY = INFINITY;
  for (int xl = 0; xl < numX; ++xl)
    for (int zl = 0; zl < numZ; ++zl) {
      const float h = hf_sample(H, heights, minX + xl, minZ + zl);
      vh[xl * numZ + zl] = h;
      maxY = fmaxf(maxY, h);
      minY = fminf(minY, h);
    }
  if (minO2 - maxY > -kHFEps) return 0;      // totally above
  if (minY - maxO2 > -kHFEps) {              // totally under
    out[0].pos[0] = g.pos[0]; out[0].pos[1] = minY; out[0].pos[2] = g.pos[2];
    out[0].normal[0] = 0.f; out[0].normal[1] = -1.f; out[0].normal[2] = 0.f;
    out[0].depth = minY - maxO2;
    kinds = kHFUnder;
    return 1;
  }
  bool further = false;
  if (g.type != G_RAY) {   // rays take the plane pass only
    const float xratio = (aabb[1] - aabb[0]) * H.inv_sw;
    if (xratio > 1.5f) further = true;
    else if ((aabb[5] - aabb[4]) * H.inv_sd > 1.5f) further = true;
  }
  // triangles: vertex indices packed as i0 | i1 << kB | i2 << 2kB | up << 3kB
  TV* tv = z.tv;
  float4* tp = z.tp;
  float* tmax = z.tmax;
  unsigned char* tstate = z.tstate;
  int numTri = 0;
  const int maxXl = maxX - minX, maxZl = maxZ - minZ;
  for (int xl = 0; xl < maxXl; ++xl) {
    for (int zl = 0; zl < maxZl; ++zl) {
      const int ia = xl * numZ + zl, ib = (xl + 1) * numZ + zl;
      const int ic = xl * numZ + zl + 1, id = (xl + 1) * numZ + zl + 1;
      const float ah = vh[ia], bh = vh[ib], ch = vh[ic], dh = vh[id];
      const bool ac = ah > minO2, bc = bh > minO2, cc = ch > minO2, dc = dh > minO2;
      vstate[ia] = !ac; vstate[ib] = !bc; vstate[ic] = !cc; vstate[id] = !dc;
      if (ac || bc || cc) {
        tv[numTri] = (TV)ia | ((TV)ib << kB) | ((TV)ic << (2 * kB)) | (TV(1) << (3 * kB));
        float m = ah > bh ? ah : bh;
        tmax[numTri] = ch > m ? ch : m;
        tstate[numTri] = 0;
        ++numTri;
      }
      if (bc || cc || dc) {
        tv[numTri] = (TV)id | ((TV)ib << kB) | ((TV)ic << (2 * kB));
        float m = dh > bh ? dh : bh;
        tmax[numTri] = ch > m ? ch : m;
        tstate[numTri] = 0;
        ++numTri;
      }
      if (further && (bc || cc) && (ah > ch && ah > bh && dh > ch && dh > bh)) {
        vstate[ib] = 1;   // concave edge BC
        vstate[ic] = 1;
      }
    }
  }
  auto vtx = [&](int i, float* v) {
    const int xl = i / numZ, zl = i - xl * numZ;
    v[0] = (minX + xl) * H.sw;
    v[1] = vh[i];
    v[2] = (minZ + zl) * H.sd;
  };
  // pass 1: planes of the triangles
  for (int k = 0; k < numTri; ++k) {
    float v0[3], v1[3], v2[3];
    vtx((int)(tv[k] & kM), v0);
    vtx((int)((tv[k] >> kB) & kM), v1);
    vtx((int)((tv[k] >> (2 * kB)) & kM), v2);
    const float e1[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
    const float e2[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
    float n[3];
    if (tv[k] >> (3 * kB)) cross3(n, e1, e2);
    else cross3(n, e2, e1);
    const float il = 1.0f / sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] *= il; n[1] *= il; n[2] *= il;
    tp[k] = make_float4(n[0], n[1], n[2], dot3(n, v0));
  }
  // group by equal plane definition, in triangle order: triangle k, when no
  // earlier plane took it, leads a plane and takes every later untaken
  // triangle whose plane matches within dEpsilon in all four components
  // (heightfield.cpp:1387-1440). Those candidates lie within dEpsilon of k's
  // offset, so they are found in a window of the triangles sorted by offset
  // instead of by a scan of every later triangle; a leader's matches are then
  // put back in triangle order.
  Idx* members = z.members;             // triangles, grouped by plane
  Idx* pfirst = z.pfirst;
  Idx* pcount = z.pcount;
  float* pmax = z.pmax;
  Idx* porder = z.porder;               // planes in sorted order
  Idx* tord = z.tord;
  Idx* trank = z.trank;
  for (int k = 0; k < numTri; ++k) tord[k] = (Idx)k;
  {
    // Shell sort by offset (Ciura's gaps); the order among equal offsets does
    // not matter: every one of them lies in the window
    const int gaps[12] = {19930, 8858, 3937, 1750, 701, 301, 132, 57, 23, 10, 4, 1};
    for (int gi = 0; gi < 12; ++gi) {
      const int gap = gaps[gi];
      for (int i = gap; i < numTri; ++i) {
        const Idx cur = tord[i];
        const float key = tp[cur].w;
        int j = i;
        while (j >= gap && tp[tord[j - gap]].w > key) {
          tord[j] = tord[j - gap];
          j -= gap;
        }
        tord[j] = cur;
      }
    }
  }
  for (int i = 0; i < numTri; ++i) trank[tord[i]] = (Idx)i;
  int numPlanes = 0, nmem = 0;
  for (int k = 0; k < numTri; ++k) {
    if (tstate[k]) continue;
    const float4 b = tp[k];
    pfirst[numPlanes] = (Idx)nmem;
    members[nmem++] = (Idx)k;
    const int first_match = nmem;
    auto take = [&](int m) {
      if (m <= k || tstate[m]) return;
      const float4 t = tp[m];
      if (fabsf(b.y - t.y) < kHFEps && fabsf(b.x - t.x) < kHFEps && fabsf(b.z - t.z) < kHFEps)
        members[nmem++] = (Idx)m;
    };
    for (int j = (int)trank[k] - 1; j >= 0 && b.w - tp[tord[j]].w < kHFEps; --j) take(tord[j]);
    for (int j = (int)trank[k] + 1; j < numTri && tp[tord[j]].w - b.w < kHFEps; ++j) take(tord[j]);
    // the matches in triangle order (the reference appends them as it scans)
    for (int i = first_match + 1; i < nmem; ++i) {
      const Idx cur = members[i];
      int j = i;
      while (j > first_match && members[j - 1] > cur) {
        members[j] = members[j - 1];
        --j;
      }
      members[j] = cur;
    }
    float mx = tmax[k];
    for (int i = first_match; i < nmem; ++i) {
      const int m = members[i];
      tstate[m] = 1;
      if (tmax[m] > mx) mx = tmax[m];
    }
    tstate[k] = 1;
    pcount[numPlanes] = (Idx)(nmem - first_match + 1);
    pmax[numPlanes] = mx;
    porder[numPlanes] = (Idx)numPlanes;
    ++numPlanes;
  }
  // sortPlanes (heightfield.cpp:910-932) bubble-sorts the planes, swapping
  // neighbours whose first height exceeds the second by more than dEpsilon.
  // A stable merge sort with the same test (the right head goes first only
  // when the left head is higher by more than dEpsilon) yields the same order
  // whenever heights are equal or further apart than dEpsilon, in
  // O(n log n) comparisons.
  {
    Idx* src = porder;
    Idx* dst = tord;                    // free once the planes are grouped
    for (int width = 1; width < numPlanes; width *= 2) {
      for (int lo = 0; lo < numPlanes; lo += 2 * width) {
        const int mid = min(lo + width, numPlanes), hi = min(lo + 2 * width, numPlanes);
        int i = lo, j = mid, o = lo;
        while (i < mid && j < hi) {
          if (pmax[src[i]] - pmax[src[j]] > kHFEps) dst[o++] = src[j++];
          else dst[o++] = src[i++];
        }
        while (i < mid) dst[o++] = src[i++];
        while (j < hi) dst[o++] = src[j++];
      }
      Idx* t = src;
      src = dst;
      dst = t;
    }
    if (src != porder)
      for (int i = 0; i < numPlanes; ++i) porder[i] = src[i];
  }
  int nc = 0;
  const unsigned plane_flags = (flags & ~0xffffu) | kHFMaxcPerCell;
  GeomView pl;
  pl.type = G_PLANE;
  for (int k = 0; k < numPlanes; ++k) {
    const int P = porder[k];
    const float4 pd = tp[members[pfirst[P]]];
    pl.p[0] = pd.x; pl.p[1] = pd.y; pl.p[2] = pd.z; pl.p[3] = pd.w;
    Contact pc[4];   // the plane colliders return at most 4 contacts
    const int npc = geom_plane_collide(g, pl, plane_flags, pc);
    bool did = false;
    for (int i = 0; i < npc; ++i) {
      for (int bq = 0; bq < pcount[P]; ++bq) {
        const int t = members[pfirst[P] + bq];
        const int i0 = (int)(tv[t] & kM);
        float corner[3];
        vtx(i0, corner);
        const int xl = i0 / numZ, zl = i0 - xl * numZ;
        if (hf_on_triangle(H, corner, minX + xl, minZ + zl, pc[i].pos, (tv[t] >> (3 * kB)) != 0)) {
          Contact& o = out[nc];
          for (int q = 0; q < 3; ++q) { o.pos[q] = pc[i].pos[q]; o.normal[q] = -pl.p[q]; }
          o.depth = pc[i].depth;
          if (++nc == max_contacts) return nc;
          did = true;
          break;
        }
      }
    }
    for (int bq = 0; bq < pcount[P]; ++bq) {
      const int t = members[pfirst[P] + bq];
      if (did) {
        vstate[tv[t] & kM] = 1;
        vstate[(tv[t] >> kB) & kM] = 1;
        vstate[(tv[t] >> (2 * kB)) & kM] = 1;
      } else {
        tstate[t] = 0;
      }
    }
  }
  // pass 2: triangle vertices against the geom's point depth
  if (further) {
    for (int k = 0; k < numTri; ++k) {
      if (tstate[k]) continue;
      for (int i = 0; i < 3; ++i) {
        const int vi = (int)((tv[k] >> (kB * i)) & kM);
        if (vstate[vi]) continue;
        float v[3];
        vtx(vi, v);
        float depth;
        bool hit;
        if (g.type == G_CYLINDER) {
          // no point-depth function for cylinders: a ray from the vertex along
          // the triangle's normal, of length (minO2 - y) * 1000, gives the
          // depth (heightfield.cpp:1562-1584)
          GeomView ray;
          ray.type = G_RAY;
          ray.pos[0] = v[0]; ray.pos[1] = v[1]; ray.pos[2] = v[2];
          for (int q = 0; q < 12; ++q) ray.R[q] = 0.f;
          ray.R[2] = tp[k].x; ray.R[6] = tp[k].y; ray.R[10] = tp[k].z;
          ray.p[0] = (minO2 - v[1]) * 1000.0f;
          ray.p[1] = ray.p[2] = ray.p[3] = 0.f;
          Contact rc;
          hit = collide_ray_cylinder(ray, g, &rc) != 0;
          depth = rc.depth;
        } else {
          depth = geom_point_depth(g, v);
          hit = depth > kHFEps;
        }
        if (hit) {
          Contact& o = out[nc];
          o.pos[0] = v[0]; o.pos[1] = v[1]; o.pos[2] = v[2];
          o.normal[0] = -tp[k].x; o.normal[1] = -tp[k].y; o.normal[2] = -tp[k].z;
          o.depth = depth;
          kinds |= kHFVertex << (2 * nc);
          if (++nc == max_contacts) return nc;
          vstate[vi] = 1;
        }
      }
    }
  }
  return nc;
}

// dCollideHeightfield(hf, g): placeable heightfield, centred origin. Returns
// the contact count (normals as the reference: pointing into the field), or
// -1 when the zone under the geom exceeds both the lane's arrays (kHFZone
// samples per axis) and the workspace `big` (none by default).
__device__ __noinline__ int collide_heightfield(const DevHeightfield& H, const float* heights, const GeomView& g,
                                               unsigned flags, Contact* out, unsigned* kinds,
                                               HFBig big = HFBig{nullptr, 0}) {
  const int maxc = (int)(flags & 0xffff);
  if (kinds) *kinds = 0u;
  if (maxc < 1) return 0;
  const float p0[3] = {g.pos[0] - H.pos[0], g.pos[1] - H.pos[1], g.pos[2] - H.pos[2]};
  GeomView g2 = g;
  mul1_331(g2.pos, H.R, p0);
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j)
      g2.R[i * 4 + j] = H.R[0 * 4 + i] * g.R[0 * 4 + j] + H.R[1 * 4 + i] * g.R[1 * 4 + j] +
                        H.R[2 * 4 + i] * g.R[2 * 4 + j];
    g2.R[i * 4 + 3] = 0.f;
  }
  g2.pos[0] += H.half_w;
  g2.pos[2] += H.half_d;
  float aabb[6];
  geom_aabb(g2, aabb);
  const bool wrapped = H.wrap != 0;
  if (!wrapped) {
    if (aabb[0] > H.width || aabb[4] > H.depth) return 0;
    if (aabb[1] < 0.f || aabb[5] < 0.f) return 0;
  }
  int nMinX = (int)floorf(nextafterf(aabb[0] * H.inv_sw, -INFINITY));
  int nMaxX = (int)ceilf(nextafterf(aabb[1] * H.inv_sw, INFINITY));
  int nMinZ = (int)floorf(nextafterf(aabb[4] * H.inv_sd, -INFINITY));
  int nMaxZ = (int)ceilf(nextafterf(aabb[5] * H.inv_sd, INFINITY));
  if (!wrapped) {
    nMinX = nMinX > 0 ? nMinX : 0;
    nMaxX = nMaxX < H.nx - 1 ? nMaxX : H.nx - 1;
    nMinZ = nMinZ > 0 ? nMinZ : 0;
    nMaxZ = nMaxZ < H.nz - 1 ? nMaxZ : H.nz - 1;
  }
  const int numX = nMaxX - nMinX + 1, numZ = nMaxZ - nMinZ + 1;
  if (numX < 1 || numZ < 1) return -1;
  unsigned kd = 0u;
  int n;
  if (numX <= kHFZone && numZ <= kHFZone) {
    HFLocalZone z;
    n = hf_zone(z, H, heights, nMinX, nMaxX, nMinZ, nMaxZ, g2, aabb, maxc, flags, out, kd);
  } else if (big.ws && numX <= big.side && numZ <= big.side) {
    HFGlobalZone z = carve_hf_ws(big.ws, big.side);
    n = hf_zone(z, H, heights, nMinX, nMaxX, nMinZ, nMaxZ, g2, aabb, maxc, flags, out, kd);
  } else {
    return -1;
  }
  if (kinds) *kinds = kd;
  for (int i = 0; i < n; ++i) {
    const float q[3] = {out[i].pos[0] - H.half_w, out[i].pos[1], out[i].pos[2] - H.half_d};
    float w[3];
    mul0_331(w, H.R, q);
    for (int k = 0; k < 3; ++k) out[i].pos[k] = w[k] + H.pos[k];
    const float nn[3] = {out[i].normal[0], out[i].normal[1], out[i].normal[2]};
    mul0_331(out[i].normal, H.R, nn);
  }
  return n;
}

}  // namespace og
