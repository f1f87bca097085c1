// sor.cuh -- the level schedule of SOR_LCP (ode/src/quickstep.cpp:342-584)
// that the adjoint replays and reverses, one warp per world (the forward step
// schedules with sor_fwd.cuh; any valid schedule gives the same sweep).
//
// The reference sweeps the rows strictly in order. Here the sweep order of an
// iteration (the concatenation of every island's current order) is turned into
// dependency levels once per reshuffle: the level of a row is one more than the
// level of the last earlier row that shares a body with it (a per-body "last
// level" carries along the sequence). Rows of one level touch disjoint bodies,
// so they run in parallel, and every body still receives its updates in the
// reference's sequence order; a friction row reads lambda[findex] at the same
// point as in the reference because it shares its bodies with its normal row.
// Rows are bucketed by level and each level is cut into chunks of 32 lanes.
#pragma once
#include "world_step.cuh"

namespace og {

struct SorSmem {
  float* fc;          // [(kMaxB+1)*6] constraint force accumulator (cforce);
                      //             slot kMaxB stays zero (second body of
                      //             one-body rows and idle lanes)
  float* lambda;      // [kMaxR+1]   entry kMaxR: idle lanes
  uint16_t* seq;      // [kMaxR]     sweep order (rows)
  uint16_t* lstart;   // [kMaxR+2]   per-level counts, then first exec slot
  uint16_t* exec;     // [kMaxR]     rows bucketed by level
  uint16_t* chunk;    // [kMaxR+32]  level of each sweep position while
                      //             scheduling, then the chunk list:
                      //             first exec slot | (count - 1) << 11
  int* last;          // [kMaxB]     last level that touched each body
};
// 13.8 KB: 16 warps per SM, matching the register limit of the kernel
constexpr int kSorSmemPerWarp = align16((kMaxB + 1) * 6 * 4 + (kMaxR + 4) * 4 + kMaxR * 2 + (kMaxR + 2) * 2 +
                                        kMaxR * 2 + (kMaxR + 32) * 2 + kMaxB * 4 + 16);
static_assert(kSorSmemPerWarp % 16 == 0, "per-warp slices must stay aligned");

OG_D SorSmem carve_sor(unsigned char* base) {
  SorSmem s;
  unsigned char* p = base;
  s.fc = reinterpret_cast<float*>(p); p += (kMaxB + 1) * 6 * 4;
  s.lambda = reinterpret_cast<float*>(p); p += (kMaxR + 4) * 4;
  s.last = reinterpret_cast<int*>(p); p += kMaxB * 4;
  s.seq = reinterpret_cast<uint16_t*>(p); p += kMaxR * 2;
  s.lstart = reinterpret_cast<uint16_t*>(p); p += (kMaxR + 2) * 2;
  s.exec = reinterpret_cast<uint16_t*>(p); p += kMaxR * 2;
  s.chunk = reinterpret_cast<uint16_t*>(p);
  return s;
}

// 16-bit counters in shared memory, updated through their 32-bit word
// (values stay far below 2^16: at most kMaxR rows).
OG_D void add_u16(uint16_t* a, int i, unsigned v) {
  unsigned* w = reinterpret_cast<unsigned*>(a + (i & ~1));
  atomicAdd(w, v << (16 * (i & 1)));
}

OG_D void row_bodies(const float* rows, int r, int& b1, int& b2) {
  const int* ri = reinterpret_cast<const int*>(rows + (size_t)r * kRowWords);
  b1 = ri[kRowB1];
  b2 = ri[kRowB2];
}

// Levels of the whole sweep sequence, then bucketing into exec/lstart.
// Returns the number of levels.
OG_D int sor_schedule(const float* rows, int nb, const SorSmem& S, int M, int lane) {
  for (int b = lane; b < nb; b += 32) S.last[b] = -1;
  for (int i = lane; i < M + 2; i += 32) S.lstart[i] = 0;
  __syncwarp();
  int nlev = 0;
  for (int base = 0; base < M; base += 32) {
    const int pos = base + lane;
    int b1 = -3, b2 = -4, level = 0;
    if (pos < M) {
      row_bodies(rows, S.seq[pos], b1, b2);
      level = S.last[b1] + 1;
      if (b2 >= 0) level = max(level, S.last[b2] + 1);
    }
#pragma unroll 4
    for (int k = 0; k < 31; ++k) {
      const int kb1 = __shfl_sync(kFull, b1, k);
      const int kb2 = __shfl_sync(kFull, b2, k);
      const int kl = __shfl_sync(kFull, level, k);
      if (lane > k) {
        const bool share = (b1 == kb1) || (b1 == kb2) || (b2 >= 0 && (b2 == kb1 || b2 == kb2));
        if (share && kl + 1 > level) level = kl + 1;
      }
    }
    __syncwarp();
    if (pos < M) {
      S.chunk[pos] = (uint16_t)level;
      add_u16(S.lstart, level, 1u);
      // rows that share a body have strictly increasing levels along the
      // sequence, so the per-body maximum is the carry for later windows
      atomicMax(&S.last[b1], level);
      if (b2 >= 0) atomicMax(&S.last[b2], level);
    }
    nlev = max(nlev, warp_max(pos < M ? level + 1 : 0));
    __syncwarp();
  }
  // exclusive prefix over the level counts -> first slot of each level
  {
    int carry = 0;
    for (int base = 0; base <= nlev; base += 32) {
      const int l = base + lane;
      const int c = (l < nlev) ? (int)S.lstart[l] : 0;
      const int incl = warp_incl_scan(c, lane);
      __syncwarp();
      if (l <= nlev) S.lstart[l] = (uint16_t)(carry + incl - c);
      carry += __shfl_sync(kFull, incl, 31);
      __syncwarp();
    }
  }
  __syncwarp();
  // scatter (order inside a level does not matter: its rows are independent);
  // lstart[l] is advanced as slots are taken and restored afterwards
  for (int pos = lane; pos < M; pos += 32) {
    const int l = S.chunk[pos];
    unsigned* w = reinterpret_cast<unsigned*>(S.lstart + (l & ~1));
    const unsigned old = atomicAdd(w, 1u << (16 * (l & 1)));
    const int slot = (int)((old >> (16 * (l & 1))) & 0xffffu);
    S.exec[slot] = S.seq[pos];
  }
  __syncwarp();
  // lstart[l] now holds the end of level l = the start of level l+1: shift back
  for (int base = ((nlev + 31) / 32) * 32; base >= 0; base -= 32) {
    const int l = base + lane;
    const uint16_t prev = (l >= 1 && l <= nlev) ? S.lstart[l - 1] : 0;
    __syncwarp();
    if (l >= 1 && l <= nlev) S.lstart[l] = prev;
    __syncwarp();
  }
  if (lane == 0) S.lstart[0] = 0;
  __syncwarp();
  // chunk list: each level split into runs of at most 32 rows
  {
    int carry = 0;
    for (int base = 0; base < nlev; base += 32) {
      const int l = base + lane;
      int a = 0, n = 0, c = 0;
      if (l < nlev) {
        a = S.lstart[l];
        n = S.lstart[l + 1] - a;
        c = (n + 31) >> 5;
      }
      const int incl = warp_incl_scan(c, lane);
      int k = carry + incl - c;
      for (int q = 0; q < c; ++q, ++k) {
        const int cnt = min(32, n - 32 * q);
        S.chunk[k] = (uint16_t)((a + 32 * q) | ((cnt - 1) << 11));
      }
      carry += __shfl_sync(kFull, incl, 31);
    }
    __syncwarp();
    return carry;   // number of chunks
  }
}

OG_D void load_row(const float* rows, int r, float4 (&rw)[8]) {
  const float4* src = reinterpret_cast<const float4*>(rows + (size_t)r * kRowWords);
#pragma unroll
  for (int q = 0; q < 8; ++q) rw[q] = __ldg(src + q);
}

}  // namespace og
