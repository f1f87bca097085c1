// sor.cuh -- SOR_LCP (ode/src/quickstep.cpp:342-584) for one world, one warp.
//
// The reference sweeps the rows strictly in order. Here the sweep order of an
// iteration (the concatenation of every island's current order) is turned into
// dependency levels once per reshuffle: the level of a row is one more than the
// level of the last earlier row that shares a body with it (a per-body "last
// level" carries along the sequence). Rows of one level touch disjoint bodies,
// so they run in parallel, and every body still receives its updates in the
// reference's sequence order; a friction row reads lambda[findex] at the same
// point as in the reference because it shares its bodies with its normal row.
// Rows are bucketed by level and each level is processed in chunks of 32 lanes,
// with the next chunk's rows (one 128-byte line each) loaded while the current
// chunk computes.
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

// One projected Gauss-Seidel row update (quickstep.cpp:484-582) on row data
// held in registers; fc and lambda live in shared memory. Written without
// branches so the lanes of a chunk never diverge: a missing second body reads
// the zero slot kMaxB (its J and iMJ halves are zero) and is not written back,
// and the friction bound is selected rather than branched on.
OG_D void sor_row(const float4 (&rw)[8], int r, const SorSmem& S) {
  const float* J = reinterpret_cast<const float*>(&rw[0]);
  const float* iMJ = reinterpret_cast<const float*>(&rw[3]);
  const float bb = rw[6].x, Ad = rw[6].y, lo = rw[6].z, hi = rw[6].w;
  const int findex = __float_as_int(rw[7].x);
  const int b1 = __float_as_int(rw[7].y), b2 = __float_as_int(rw[7].z);
  const bool two = b2 >= 0;
  float* fc1 = S.fc + 6 * b1;
  float* fc2 = S.fc + 6 * (two ? b2 : kMaxB);
  const float old = S.lambda[r];
  const float lf = S.lambda[findex >= 0 ? findex : kMaxR];
  const float f10 = fc1[0], f11 = fc1[1], f12 = fc1[2], f13 = fc1[3], f14 = fc1[4], f15 = fc1[5];
  const float f20 = fc2[0], f21 = fc2[1], f22 = fc2[2], f23 = fc2[3], f24 = fc2[4], f25 = fc2[5];
  float delta = bb - old * Ad;
  // the 6-term dot products are summed pairwise (shorter dependency chains
  // than the reference's left-to-right sums; same terms)
  delta -= (f10 * J[0] + f11 * J[1]) + (f12 * J[2] + f13 * J[3]) + (f14 * J[4] + f15 * J[5]);
  delta -= (f20 * J[6] + f21 * J[7]) + (f22 * J[8] + f23 * J[9]) + (f24 * J[10] + f25 * J[11]);
  const float hf = fabsf(hi * lf);
  const float hi_act = findex >= 0 ? hf : hi;
  const float lo_act = findex >= 0 ? -hf : lo;
  const float nl = old + delta;
  // the reference keeps delta when no bound is hit and uses bound - old otherwise
  const bool clamped = (nl < lo_act) || (nl > hi_act);
  const float lam = fminf(fmaxf(nl, lo_act), hi_act);
  delta = clamped ? lam - old : delta;
  S.lambda[r] = clamped ? lam : nl;
  fc1[0] = f10 + delta * iMJ[0]; fc1[1] = f11 + delta * iMJ[1]; fc1[2] = f12 + delta * iMJ[2];
  fc1[3] = f13 + delta * iMJ[3]; fc1[4] = f14 + delta * iMJ[4]; fc1[5] = f15 + delta * iMJ[5];
  if (two) {
    fc2[0] = f20 + delta * iMJ[6]; fc2[1] = f21 + delta * iMJ[7]; fc2[2] = f22 + delta * iMJ[8];
    fc2[3] = f23 + delta * iMJ[9]; fc2[4] = f24 + delta * iMJ[10]; fc2[5] = f25 + delta * iMJ[11];
  }
}

// Row data of an idle lane: no effect (zero J and iMJ, bounds 0, first body is
// the zero slot, lambda slot kMaxR).
OG_D void idle_row(float4 (&rw)[8]) {
#pragma unroll
  for (int q = 0; q < 7; ++q) rw[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  rw[7] = make_float4(__int_as_float(-1), __int_as_float(kMaxB), __int_as_float(-1), 0.f);
}

OG_D void load_row(const float* rows, int r, float4 (&rw)[8]) {
  const float4* src = reinterpret_cast<const float4*>(rows + (size_t)r * kRowWords);
#pragma unroll
  for (int q = 0; q < 8; ++q) rw[q] = __ldg(src + q);
}

// SOR over every island of the world. island_rstart: [nisl+1] world rows.
// Returns the RNG state after the step (the islands' shuffles consume ODE's
// stream in island order, ceil(iters/8) * (m - 1) draws each).
OG_D unsigned sor_world(const float* rows, const int* rstart, int nb, int M, int nisl, int iters,
                        unsigned seed, const SorSmem& S, int lane) {
  for (int i = lane; i < nb * 6; i += 32) S.fc[i] = 0.f;
  if (lane < 6) S.fc[kMaxB * 6 + lane] = 0.f;
  for (int i = lane; i < M; i += 32) S.lambda[i] = 0.f;
  if (lane == 0) S.lambda[kMaxR] = 0.f;
  const int n_shuffles = (iters + 7) / 8;
  // initial order per island: findex == -1 rows first (ascending), the rest
  // from the island's tail backwards (quickstep.cpp:405-425)
  for (int isl = 0; isl < nisl; ++isl) {
    const int rs = rstart[isl], re = rstart[isl + 1];
    int negc = 0;
    for (int base = rs; base < re; base += 32) {
      const int r = base + lane;
      bool neg = false;
      if (r < re) neg = reinterpret_cast<const int*>(rows + (size_t)r * kRowWords)[kRowFindex] == -1;
      const unsigned bal = __ballot_sync(kFull, neg && r < re);
      const int negb = negc + __popc(bal & ((1u << lane) - 1u));
      if (r < re) {
        const int nonnegb = (r - rs) - negb;
        const int p = neg ? rs + negb : re - 1 - nonnegb;
        S.seq[p] = (uint16_t)r;
      }
      negc += __popc(bal);
    }
  }
  __syncwarp();
  unsigned total_draws = 0;
  for (int isl = 0; isl < nisl; ++isl) {
    const int m = rstart[isl + 1] - rstart[isl];
    if (m > 0) total_draws += (unsigned)(n_shuffles * (m - 1));
  }
  int nchunk = 0;
  for (int it = 0; it < iters; ++it) {
    if ((it & 7) == 0) {
      const int round = it >> 3;
      unsigned prefix = 0;
      for (int ib = 0; ib < nisl; ib += 32) {
        const int isl = ib + lane;
        int m = 0;
        if (isl < nisl) m = rstart[isl + 1] - rstart[isl];
        const int draws = m > 0 ? n_shuffles * (m - 1) : 0;
        const int incl = warp_incl_scan(draws, lane);
        if (isl < nisl && m > 1) {
          unsigned s = lcg_jump(seed, prefix + (unsigned)(incl - draws) + (unsigned)(round * (m - 1)));
          uint16_t* sq = S.seq + rstart[isl];
          for (int q = 1; q < m; ++q) {
            s = lcg_next(s);
            const int sw = rand_int_from(s, q + 1);
            const uint16_t t = sq[q];
            sq[q] = sq[sw];
            sq[sw] = t;
          }
        }
        prefix += (unsigned)__shfl_sync(kFull, incl, 31);
      }
      __syncwarp();
      nchunk = sor_schedule(rows, nb, S, M, lane);
    }
    // sweep: chunks in level order; the next chunk's rows are loaded while
    // the current one computes (two register buffers used in turn). Idle lanes
    // run a no-op row so the warp never diverges.
    float4 ra[8], rb[8];
    int r_a, r_b;
    {
      const unsigned c0 = S.chunk[0];
      r_a = kMaxR;
      if (lane <= (int)(c0 >> 11)) { r_a = S.exec[(c0 & 0x7ffu) + lane]; load_row(rows, r_a, ra); }
      else idle_row(ra);
    }
    for (int k = 0; k < nchunk; k += 2) {
      r_b = kMaxR;
      if (k + 1 < nchunk) {
        const unsigned c1 = S.chunk[k + 1];
        if (lane <= (int)(c1 >> 11)) { r_b = S.exec[(c1 & 0x7ffu) + lane]; load_row(rows, r_b, rb); }
        else idle_row(rb);
      }
      sor_row(ra, r_a, S);
      __syncwarp();
      if (k + 1 >= nchunk) break;
      r_a = kMaxR;
      if (k + 2 < nchunk) {
        const unsigned c2 = S.chunk[k + 2];
        if (lane <= (int)(c2 >> 11)) { r_a = S.exec[(c2 & 0x7ffu) + lane]; load_row(rows, r_a, ra); }
        else idle_row(ra);
      }
      sor_row(rb, r_b, S);
      __syncwarp();
    }
  }
  return lcg_jump(seed, total_draws);
}

}  // namespace og
