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

// Heightfield workspaces for a second pass over rays whose zone exceeded the
// lane's arrays: warp slot k (of the launch's warps) uses ws + k * stride.
struct RayBig {
  unsigned char* ws;
  long long stride;
  int side;
};

// hits[i].geom: the world-local geom index, -1 when nothing is hit, -2 for an
// invalid ray (world or body out of range, bad length); -3 when a heightfield
// zone under the ray exceeds the lane's arrays and the launch has no
// workspace (or the workspace's side). `list` (optional) names the rays to
// cast; each warp casts rays slot, slot + warps, ... of it.
__global__ void __launch_bounds__(128) raycast_kernel(BatchDev d, const odegpuRay* rays, const int* list, int n,
                                                      unsigned flags, odegpuRayHit* hits, RayBig big) {
  const int lane = threadIdx.x & 31;
  const int slot = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const HFBig hb{big.ws ? big.ws + (size_t)slot * big.stride : nullptr, big.side};
  for (int k = slot; k < n; k += warps) {
    const int i = list ? list[k] : k;
    const odegpuRay r = rays[i];
    odegpuRayHit h;
    h.geom = -1;
    h.pos[0] = h.pos[1] = h.pos[2] = 0.f;
    h.normal[0] = h.normal[1] = h.normal[2] = 0.f;
    h.depth = 0.f;
    if (r.world < 0 || r.world >= d.n_worlds) {
      h.geom = -2;
      if (lane == 0) hits[i] = h;
      continue;
    }
    const WorldDesc D = d.world[r.world];
    GeomView rv;
    if (!ray_view(d, D, r, rv)) {
      h.geom = -2;
      if (lane == 0) hits[i] = h;
      continue;
    }
    float best = INFINITY;
    int bg = 0x7fffffff;
    bool zone = false;
    Contact bc;
    for (int g0 = 0; g0 < D.ng; g0 += 32) {
      const int g = g0 + lane;
      int cnt = 0;
      Contact cc[8];
      bool hf = false;
      if (g < D.ng && !(r.body >= 0 && d.gbody[D.geom_off + g] == r.body)) {   // geoms on one body (collision_kernel.cpp:296-303)
        GeomView gv;
        geom_view(d, D, g, gv);
        if (gv.type == G_HEIGHTFIELD) {
          // dCollide(ray, field): the field collides first, normals negated
          hf = true;
          cnt = collide_heightfield(d.hfs[(int)gv.p[0]], d.hf_heights, rv, flags, cc, nullptr);
        } else {
          cnt = collide_primitive(rv, gv, flags, cc);
        }
      }
      // zones beyond the lane's arrays: the lanes take turns on the warp's workspace
      if (hb.ws) {
        unsigned todo = __ballot_sync(kFull, hf && cnt < 0);
        while (todo) {
          const int l = __ffs(todo) - 1;
          todo &= todo - 1;
          if (lane == l) {
            GeomView gv;
            geom_view(d, D, g, gv);
            cnt = collide_heightfield(d.hfs[(int)gv.p[0]], d.hf_heights, rv, flags, cc, nullptr, hb);
          }
          __syncwarp();
        }
      }
      if (cnt < 0) { zone = true; cnt = 0; }
      if (hf)
        for (int c = 0; c < cnt; ++c) {
          cc[c].normal[0] = -cc[c].normal[0]; cc[c].normal[1] = -cc[c].normal[1]; cc[c].normal[2] = -cc[c].normal[2];
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
      continue;
    }
    if (wg != 0x7fffffff && bg == wg) {   // the lane that holds the winner writes it
      h.geom = wg;
      for (int q = 0; q < 3; ++q) { h.pos[q] = bc.pos[q]; h.normal[q] = bc.normal[q]; }
      h.depth = bc.depth;
      hits[i] = h;
    } else if (wg == 0x7fffffff && lane == 0) {
      hits[i] = h;
    }
  }
}

}  // namespace og
