// raycast.cuh -- batched ray queries against the worlds of a batch.
//
// ODE answers a ray query with a ray geom (dRayClass, ode/src/ray.cpp) and
// dSpaceCollide2(ray, space, ...): the space hands every geom whose bounding
// box meets the ray's to the callback, which calls dCollide(ray, geom) and
// usually keeps the nearest contact. Bounding boxes only cull, so the nearest
// contact equals the least-depth contact of dCollide(ray, g) over every geom g
// of the world; that is what this kernel computes, one warp per ray, lanes
// striding over the world's geoms, the winner picked by a warp reduction
// (least depth, then the lower geom index).
#pragma once
#include "odegpu.h"
#include "world_step.cuh"

namespace og {

// The ray as a geom view: start and direction placed with the body's pose when
// the ray is attached (a geom offset: final pos = pos_b + R_b start, direction
// = R_b dir, ode/src/collision_kernel.cpp dxGeom::computePosr).
OG_D bool ray_view(const BatchDev& d, const WorldDesc& D, const odegpuRay& r, GeomView& v) {
  float dir[3] = {r.dir[0], r.dir[1], r.dir[2]};
  safe_normalize3(dir);   // dGeomRaySet normalises (ray.cpp:115-136)
  v.type = G_RAY;
  v.p[0] = r.length; v.p[1] = v.p[2] = v.p[3] = 0.f;
  for (int k = 0; k < 12; ++k) v.R[k] = 0.f;
  if (r.body >= 0) {
    if (r.body >= D.nb) return false;
    float R[12];
    body_R(d, D.body_off + r.body, R);
    const float4 ps = d.pos[D.body_off + r.body];
    float s[3], w[3];
    mul0_331(s, R, r.start);
    mul0_331(w, R, dir);
    v.pos[0] = ps.x + s[0]; v.pos[1] = ps.y + s[1]; v.pos[2] = ps.z + s[2];
    v.R[2] = w[0]; v.R[6] = w[1]; v.R[10] = w[2];
  } else {
    for (int k = 0; k < 3; ++k) v.pos[k] = r.start[k];
    v.R[2] = dir[0]; v.R[6] = dir[1]; v.R[10] = dir[2];
  }
  return isfinite(r.length) && r.length >= 0.f;
}

// hits[i].geom: the world-local geom index, -1 when nothing is hit, -2 for an
// invalid ray (world or body out of range, bad length); -3 when a heightfield
// zone under the ray exceeds the collider's lane buffers.
__global__ void __launch_bounds__(128) raycast_kernel(BatchDev d, const odegpuRay* rays, int n, unsigned flags,
                                                      odegpuRayHit* hits) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= n) return;
  const odegpuRay r = rays[i];
  odegpuRayHit h;
  h.geom = -1;
  h.pos[0] = h.pos[1] = h.pos[2] = 0.f;
  h.normal[0] = h.normal[1] = h.normal[2] = 0.f;
  h.depth = 0.f;
  if (r.world < 0 || r.world >= d.n_worlds) {
    h.geom = -2;
    if (lane == 0) hits[i] = h;
    return;
  }
  const WorldDesc D = d.world[r.world];
  GeomView rv;
  if (!ray_view(d, D, r, rv)) {
    h.geom = -2;
    if (lane == 0) hits[i] = h;
    return;
  }
  float best = INFINITY;
  int bg = 0x7fffffff;
  bool zone = false;
  Contact bc;
  for (int g = lane; g < D.ng; g += 32) {
    const int gg = D.geom_off + g;
    if (r.body >= 0 && d.gbody[gg] == r.body) continue;   // geoms on one body (collision_kernel.cpp:296-303)
    GeomView gv;
    geom_view(d, D, g, gv);
    Contact cc[8];
    int cnt;
    if (gv.type == G_HEIGHTFIELD) {
      // dCollide(ray, field): the field collides first, normals negated
      cnt = collide_heightfield(d.hfs[(int)gv.p[0]], d.hf_heights, rv, flags, cc, nullptr);
      if (cnt < 0) { zone = true; cnt = 0; }
      for (int c = 0; c < cnt; ++c) {
        cc[c].normal[0] = -cc[c].normal[0]; cc[c].normal[1] = -cc[c].normal[1]; cc[c].normal[2] = -cc[c].normal[2];
      }
    } else {
      cnt = collide_primitive(rv, gv, flags, cc);
    }
    for (int c = 0; c < cnt; ++c)
      if (cc[c].depth < best) { best = cc[c].depth; bg = g; bc = cc[c]; }
  }
  // least depth, then the lower geom index
  float wd = best;
  int wg = bg;
  for (int o = 16; o > 0; o >>= 1) {
    const float od = __shfl_xor_sync(kFull, wd, o);
    const int og_ = __shfl_xor_sync(kFull, wg, o);
    if (od < wd || (od == wd && og_ < wg)) { wd = od; wg = og_; }
  }
  if (__ballot_sync(kFull, zone)) {   // the nearest hit may lie in the zone not searched
    if (lane == 0) { h.geom = -3; hits[i] = h; }
    return;
  }
  if (wg != 0x7fffffff && bg == wg) {   // the lane that holds the winner writes it
    h.geom = wg;
    for (int k = 0; k < 3; ++k) { h.pos[k] = bc.pos[k]; h.normal[k] = bc.normal[k]; }
    h.depth = bc.depth;
    hits[i] = h;
  } else if (wg == 0x7fffffff && lane == 0) {
    hits[i] = h;
  }
}

}  // namespace og
