// sor_fwd.cuh -- SOR_LCP (ode/src/quickstep.cpp:342-584) of the forward step,
// one warp per world.
//
// The result is the reference's sequential projected Gauss-Seidel sweep: the
// sweep order of an iteration (every island's current order, concatenated)
// is split into dependency levels once per reshuffle (a row's level is one
// more than the level of the last earlier row that shares a body with it), so
// rows of one level touch disjoint bodies and run on the lanes in parallel,
// while every body receives its updates in the reference's sequence and a
// friction row reads lambda[findex] at the same point. Any assignment with
// that property gives bit-identical results; this one is the shortest.
//
// The kernel is bound by the L1/shared-memory data path and by the latency of
// a world's chain of dependent chunks, so the path is built to move fewer
// bytes per chunk and to wait less:
//   * levels: sixteen sequence positions per window, the two body entries of
//     each row on two lanes; __match_any_sync finds each entry's previous
//     entry on the same body, and the levels settle by relaxation in as many
//     rounds as the window's longest chain (usually 2-4), instead of 31
//     dependent shuffle rounds per 32 rows;
//   * row traffic: the first iteration of a round reads each chunk's rows
//     from the row store (one 128-byte line per lane) and writes them, in
//     execution order, into the world's sweep buffer, quad-major (quad q of
//     every slot contiguous, word 31 replaced by the row's index); the
//     round's later iterations read the buffer, where one instruction covers
//     a chunk's quads with one or two contiguous segments instead of one line
//     per lane. The next chunk's rows are loaded while a chunk computes (two
//     register buffers used in turn), and idle lanes load nothing;
//   * the per-body accumulators are one float4 and one float2 per body;
//   * the shuffle's swap targets are drawn lane-parallel (LCG jump-ahead),
//     leaving one lane per island only the swaps themselves; the island table
//     and each row's bodies and findex flag are staged in shared memory once.
// A world whose rows exceed kFwdRows keeps its row-indexed arrays (lambda,
// order, levels, chunk list, row bodies) in a per-world global scratch area;
// the code is the same, only the pointers differ.
#pragma once
#include "world_step.cuh"

namespace og {

constexpr int kFwdRows = 512;   // rows whose SOR arrays fit the warp's shared memory

struct FwdSmem {
  float* fc;          // [(kMaxB+1)*6] cforce per body after the sweep; slot kMaxB zero
  float4* fcA;        // the same bytes during the sweep: fcA[b] = cforce 0..3,
  float2* fcB;        //   fcB[b] = cforce 4..5
  int* last;          // [kMaxB] last level that touched each body (scheduling)
  int* rstart;        // [kMaxB+1] first row of each island (the step's island table)
  // row-indexed arrays: shared memory when M <= kFwdRows, else global scratch
  float* lambda;      // [cap+1]   entry cap: idle lanes
  uint16_t* seq;      // [cap]     sweep order (rows)
  uint16_t* lstart;   // [cap+2]   per-level counts, then first exec slot
  uint16_t* exec;     // [cap]     shuffle swap targets, then rows bucketed by level
  uint16_t* chunk;    // [cap+32]  level of each sweep position while scheduling,
                      //           then the chunk list: first slot | (count - 1) << 11
  uint16_t* rbody;    // [cap]     b1 | (b2 + 1) << 8, bit 15: findex == -1
  int cap;            // rows the arrays hold (kFwdRows or kMaxR)
};

constexpr int fwd_row_arrays_bytes(int cap) {
  return align16((cap + 4) * 4) + align16(cap * 2) + align16((cap + 2) * 2) + align16(cap * 2) +
         align16((cap + 32) * 2) + align16(cap * 2);
}
constexpr int kFwdSmemPerWarp = align16((kMaxB + 1) * 6 * 4) + align16(kMaxB * 4) + align16((kMaxB + 1) * 4) +
                                fwd_row_arrays_bytes(kFwdRows);
constexpr int kFwdScratchPerWorld = fwd_row_arrays_bytes(kMaxR);   // bytes, worlds with row_cap > kFwdRows
static_assert(kFwdSmemPerWarp % 16 == 0, "per-warp slices must stay aligned");

OG_D void carve_row_arrays(unsigned char* p, int cap, FwdSmem& s) {
  s.cap = cap;
  s.lambda = reinterpret_cast<float*>(p); p += align16((cap + 4) * 4);
  s.seq = reinterpret_cast<uint16_t*>(p); p += align16(cap * 2);
  s.lstart = reinterpret_cast<uint16_t*>(p); p += align16((cap + 2) * 2);
  s.exec = reinterpret_cast<uint16_t*>(p); p += align16(cap * 2);
  s.chunk = reinterpret_cast<uint16_t*>(p); p += align16((cap + 32) * 2);
  s.rbody = reinterpret_cast<uint16_t*>(p);
}

// base: the warp's kFwdSmemPerWarp bytes of shared memory; scratch: the
// world's global scratch area (null when it has none)
OG_D FwdSmem carve_fwd(unsigned char* base, int M, unsigned char* scratch) {
  FwdSmem s;
  unsigned char* p = base;
  s.fc = reinterpret_cast<float*>(p);
  s.fcA = reinterpret_cast<float4*>(p);
  s.fcB = reinterpret_cast<float2*>(p + (kMaxB + 1) * 16);
  p += align16((kMaxB + 1) * 6 * 4);
  s.last = reinterpret_cast<int*>(p); p += align16(kMaxB * 4);
  s.rstart = reinterpret_cast<int*>(p); p += align16((kMaxB + 1) * 4);
  if (M <= kFwdRows || !scratch) carve_row_arrays(p, kFwdRows, s);
  else carve_row_arrays(scratch, kMaxR, s);
  return s;
}

// 16-bit counters updated through their 32-bit word (values stay below 2^16)
OG_D void add_u16_fwd(uint16_t* a, int i, unsigned v) {
  unsigned* w = reinterpret_cast<unsigned*>(a + (i & ~1));
  atomicAdd(w, v << (16 * (i & 1)));
}

// Levels of the sweep sequence (S.seq), bucketing into S.exec, chunk list in
// S.chunk. Returns the number of chunks.
OG_D int fwd_schedule(const FwdSmem& S, int nb, int M, int lane) {
  for (int b = lane; b < nb; b += 32) S.last[b] = -1;
  for (int i = lane; i < M + 2; i += 32) S.lstart[i] = 0;
  __syncwarp();
  int nlev = 0;
  const int side = lane & 1;
  const unsigned below = (1u << lane) - 1u;
  for (int base = 0; base < M; base += 16) {
    const int pos = base + (lane >> 1);
    int body = -1;
    if (pos < M) {
      const int rb = S.rbody[S.seq[pos]];
      body = side ? ((rb >> 8) & 0x7f) - 1 : (rb & 0xff);
    }
    const bool valid = body >= 0;
    // entries without a body match nothing
    const unsigned mask = __match_any_sync(kFull, valid ? body : -1 - lane);
    const unsigned lower = mask & below;
    const int prev = lower ? 31 - __clz(lower) : lane;
    const int base_lvl = valid ? S.last[body] + 1 : 0;
    int lvl = max(base_lvl, __shfl_xor_sync(kFull, base_lvl, 1));
    for (;;) {
      const int pl = __shfl_sync(kFull, lvl, prev);
      int cand = lower ? pl + 1 : 0;
      cand = max(cand, __shfl_xor_sync(kFull, cand, 1));
      const bool up = cand > lvl;
      lvl = up ? cand : lvl;
      if (!__any_sync(kFull, up)) break;
    }
    __syncwarp();
    // the last entry of each body in the window carries its level on
    if (valid && (mask >> lane) == 1u) S.last[body] = lvl;
    if (pos < M && side == 0) {
      S.chunk[pos] = (uint16_t)lvl;
      add_u16_fwd(S.lstart, lvl, 1u);
    }
    if (pos < M) nlev = max(nlev, lvl + 1);
    __syncwarp();
  }
  nlev = warp_max(nlev);
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
  return carry;
}

// the LCG advanced by 32 calls: x -> kLcg32A x + kLcg32C (mod 2^32)
constexpr unsigned lcg_pow_a(int k) { return k == 0 ? 1u : 1664525u * lcg_pow_a(k - 1); }
constexpr unsigned lcg_pow_c(int k) { return k == 0 ? 0u : 1664525u * lcg_pow_c(k - 1) + 1013904223u; }
constexpr unsigned kLcg32A = lcg_pow_a(32);
constexpr unsigned kLcg32C = lcg_pow_c(32);

// One row update of the sweep (quickstep.cpp:484-582) on a row held in
// registers (word 31: the row's index). The arithmetic is sor_row's; lanes
// past the chunk's end (active false) read the zero body slot and the dummy
// lambda and store nothing.
OG_D void fwd_row(const float4 (&rw)[8], bool active, const FwdSmem& S) {
  const float* J = reinterpret_cast<const float*>(&rw[0]);
  const float* iMJ = reinterpret_cast<const float*>(&rw[3]);
  const float bb = rw[6].x, Ad = rw[6].y, lo = rw[6].z, hi = rw[6].w;
  const int findex = active ? __float_as_int(rw[7].x) : -1;
  const int b1 = active ? __float_as_int(rw[7].y) : kMaxB;
  const int b2r = __float_as_int(rw[7].z);
  const bool two = active && b2r >= 0;
  const int b2 = two ? b2r : kMaxB;
  const int r = active ? __float_as_int(rw[7].w) : S.cap;
  const float4 a1 = S.fcA[b1];
  const float2 c1 = S.fcB[b1];
  const float4 a2 = S.fcA[b2];
  const float2 c2 = S.fcB[b2];
  const float old = S.lambda[r];
  const float lf = S.lambda[findex >= 0 ? findex : S.cap];
  float delta = bb - old * Ad;
  // the 6-term dot products are summed pairwise (same terms as the
  // reference's left-to-right sums, shorter dependency chains)
  delta -= (a1.x * J[0] + a1.y * J[1]) + (a1.z * J[2] + a1.w * J[3]) + (c1.x * J[4] + c1.y * J[5]);
  delta -= (a2.x * J[6] + a2.y * J[7]) + (a2.z * J[8] + a2.w * J[9]) + (c2.x * J[10] + c2.y * J[11]);
  const float hf = fabsf(hi * lf);
  const float hi_act = findex >= 0 ? hf : hi;
  const float lo_act = findex >= 0 ? -hf : lo;
  const float nl = old + delta;
  // the reference keeps delta when no bound is hit and uses bound - old otherwise
  const bool clamped = (nl < lo_act) || (nl > hi_act);
  const float lam = fminf(fmaxf(nl, lo_act), hi_act);
  delta = clamped ? lam - old : delta;
  if (active) {
    S.lambda[r] = clamped ? lam : nl;
    S.fcA[b1] = make_float4(a1.x + delta * iMJ[0], a1.y + delta * iMJ[1], a1.z + delta * iMJ[2],
                            a1.w + delta * iMJ[3]);
    S.fcB[b1] = make_float2(c1.x + delta * iMJ[4], c1.y + delta * iMJ[5]);
    if (two) {
      S.fcA[b2] = make_float4(a2.x + delta * iMJ[6], a2.y + delta * iMJ[7], a2.z + delta * iMJ[8],
                              a2.w + delta * iMJ[9]);
      S.fcB[b2] = make_float2(c2.x + delta * iMJ[10], c2.y + delta * iMJ[11]);
    }
  }
}

// Rows of chunk c for this lane: from the row store (first iteration of the
// round) or from the sweep buffer; returns whether the lane has a row. Lanes
// past the chunk's end load the chunk's last row again (the same lines, no
// divergent branch) and are masked out by fwd_row.
template <bool kFirst>
OG_D bool fwd_load(const float* rows, const float4* sweep, int capp, const FwdSmem& S, unsigned c, int lane,
                   float4 (&rw)[8]) {
  const int last = (int)(c >> 11);
  const bool active = lane <= last;
  const int slot = (int)(c & 0x7ffu) + (active ? lane : last);
  if (kFirst) {
    const int r = S.exec[slot];
    const float4* src = reinterpret_cast<const float4*>(rows) + (size_t)r * 8;
#pragma unroll
    for (int q = 0; q < 8; ++q) rw[q] = src[q];
    rw[7].w = __int_as_float(r);
  } else {
#pragma unroll
    for (int q = 0; q < 8; ++q) rw[q] = sweep[(size_t)q * capp + slot];
  }
  return active;
}
// the first iteration's rows into the sweep buffer
OG_D void fwd_keep(float4* sweep, int capp, unsigned c, bool active, int lane, const float4 (&rw)[8]) {
  if (!active) return;
  const int slot = (int)(c & 0x7ffu) + lane;
#pragma unroll
  for (int q = 0; q < 8; ++q) sweep[(size_t)q * capp + slot] = rw[q];
}

// One iteration over the chunk list (S.chunk, rows of the slots in S.exec);
// the first iteration of a round reads the row store and fills the sweep
// buffer, the others read the sweep buffer.
template <bool kFirst>
OG_D void fwd_iteration(const float* rows, float4* sweep, int capp, const FwdSmem& S, int nchunk, int lane) {
  float4 ra[8], rb[8];
  unsigned ca = S.chunk[0], cb = 0;
  bool act_a = fwd_load<kFirst>(rows, sweep, capp, S, ca, lane, ra), act_b = false;
  for (int k = 0; k < nchunk; k += 2) {
    if (k + 1 < nchunk) {
      cb = S.chunk[k + 1];
      act_b = fwd_load<kFirst>(rows, sweep, capp, S, cb, lane, rb);
    }
    fwd_row(ra, act_a, S);
    if (kFirst) fwd_keep(sweep, capp, ca, act_a, lane, ra);
    __syncwarp();
    if (k + 1 >= nchunk) break;
    if (k + 2 < nchunk) {
      ca = S.chunk[k + 2];
      act_a = fwd_load<kFirst>(rows, sweep, capp, S, ca, lane, ra);
    }
    fwd_row(rb, act_b, S);
    if (kFirst) fwd_keep(sweep, capp, cb, act_b, lane, rb);
    __syncwarp();
  }
}

// n_it iterations of one reshuffle round over the chunk list.
OG_D void fwd_sweep(const float* rows, float4* sweep, int capp, const FwdSmem& S, int nchunk, int n_it, int lane) {
  if (n_it < 1 || nchunk < 1) return;
  fwd_iteration<true>(rows, sweep, capp, S, nchunk, lane);
  for (int it = 1; it < n_it; ++it) fwd_iteration<false>(rows, sweep, capp, S, nchunk, lane);
}

// SOR over every island of the world (rows of island i start at world row
// rstart_g[i]). Returns the RNG state after the step (the islands' shuffles
// consume ODE's stream in island order, ceil(iters/8) * (m - 1) draws each).
// On return S.fc holds cforce per body (six floats) and S.lambda the
// multipliers by row. sweep / capp: the world's sweep buffer and its slot
// stride (row capacity + 32).
OG_D unsigned fwd_sor_world(const float* rows, const int* rstart_g, int nb, int M, int nisl, int iters,
                            unsigned seed, const FwdSmem& S, int lane, float4* sweep, int capp) {
  for (int i = lane; i <= nisl; i += 32) S.rstart[i] = rstart_g[i];
  for (int i = lane; i < (kMaxB + 1) * 6; i += 32) S.fc[i] = 0.f;
  for (int i = lane; i < M; i += 32) S.lambda[i] = 0.f;
  if (lane == 0) S.lambda[S.cap] = 0.f;
  // each row's bodies and whether it has findex == -1
  for (int r = lane; r < M; r += 32) {
    const int4 w7 = reinterpret_cast<const int4*>(rows + (size_t)r * kRowWords)[7];   // findex b1 b2 joint
    S.rbody[r] = (uint16_t)(w7.y | ((w7.z + 1) << 8) | (w7.x == -1 ? 0x8000 : 0));
  }
  __syncwarp();
  // initial order per island: findex == -1 rows first (ascending), the rest
  // from the island's tail backwards (quickstep.cpp:405-425)
  for (int isl = 0; isl < nisl; ++isl) {
    const int rs = S.rstart[isl], re = S.rstart[isl + 1];
    int negc = 0;
    for (int base = rs; base < re; base += 32) {
      const int r = base + lane;
      const bool neg = r < re && (S.rbody[r] & 0x8000) != 0;
      const unsigned bal = __ballot_sync(kFull, neg);
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
  const int n_shuffles = (iters + 7) / 8;
  // draws of the whole step: ceil(iters / 8) (m - 1) per island
  unsigned total_draws = 0;
  for (int ib = 0; ib < nisl; ib += 32) {
    const int isl = ib + lane;
    const int m = isl < nisl ? S.rstart[isl + 1] - S.rstart[isl] : 0;
    total_draws += (unsigned)__reduce_add_sync(kFull, (unsigned)(m > 0 ? n_shuffles * (m - 1) : 0));
  }
  for (int it = 0; it < iters; it += 8) {
    const int round = it >> 3;
    // the round's swap targets, dRandInt(q + 1) for step q = 1 .. m - 1 of
    // each island's shuffle (quickstep.cpp:471-478). ODE draws them island by
    // island, every round of an island before the next island, so draw q of
    // island i in this round is the seed advanced by base_i + round (m_i - 1)
    // + q, base_i the draws of the islands before it. The round's (island, q)
    // entries are cut into one contiguous run per lane: a jump-ahead to the
    // run's first entry, then one LCG step per entry. The island tables live
    // in S.last and S.lstart until fwd_schedule claims them.
    {
      int* iex = S.last;                                        // entries before island i
      unsigned* ist = reinterpret_cast<unsigned*>(S.lstart);    // seed before island i's round
      int T = 0;
      unsigned base = 0;
      for (int ib = 0; ib < nisl; ib += 32) {
        const int isl = ib + lane;
        const int m = isl < nisl ? S.rstart[isl + 1] - S.rstart[isl] : 0;
        const int e = m > 1 ? m - 1 : 0;
        const int d = n_shuffles * e;
        const int incl_e = warp_incl_scan(e, lane);
        const int incl_d = warp_incl_scan(d, lane);
        if (isl < nisl) {
          iex[isl] = T + incl_e - e;
          ist[isl] = lcg_jump(seed, base + (unsigned)(incl_d - d) + (unsigned)(round * e));
        }
        T += __shfl_sync(kFull, incl_e, 31);
        base += (unsigned)__shfl_sync(kFull, incl_d, 31);
      }
      __syncwarp();
      const int per = (T + 31) >> 5;
      const int e0 = lane * per, e1 = min(T, e0 + per);
      if (e0 < e1) {
        // the island of entry e0: the last island whose first entry is <= e0
        int lo = 0, hi = nisl - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (iex[mid] <= e0) lo = mid;
          else hi = mid - 1;
        }
        int i = lo, r0 = S.rstart[i], m = S.rstart[i + 1] - r0, q = e0 - iex[i] + 1;
        unsigned sd = lcg_jump(ist[i], (unsigned)q);
        for (int e = e0;;) {
          S.exec[r0 + q] = (uint16_t)rand_int_from(sd, q + 1);
          if (++e >= e1) break;
          if (++q < m) {
            sd = lcg_next(sd);
            continue;
          }
          do {                       // the next island with draws
            ++i;
            r0 = S.rstart[i];
            m = S.rstart[i + 1] - r0;
          } while (m <= 1);
          q = 1;
          sd = lcg_next(ist[i]);
        }
      }
    }
    __syncwarp();
    // the swaps themselves, one lane per island, in the reference's order
    for (int isl = lane; isl < nisl; isl += 32) {
      const int r0 = S.rstart[isl], m = S.rstart[isl + 1] - r0;
      uint16_t* sq = S.seq + r0;
      const uint16_t* sw = S.exec + r0;
      for (int q = 1; q < m; ++q) {
        const int k = sw[q];
        const uint16_t t = sq[q];
        sq[q] = sq[k];
        sq[k] = t;
      }
    }
    __syncwarp();
    const int nchunk = fwd_schedule(S, nb, M, lane);
    fwd_sweep(rows, sweep, capp, S, nchunk, min(8, iters - it), lane);
  }
  // cforce back to six floats per body
  {
    float4 a[2];
    float2 c[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int b = lane + 32 * h;
      if (b < nb) { a[h] = S.fcA[b]; c[h] = S.fcB[b]; }
    }
    __syncwarp();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int b = lane + 32 * h;
      if (b < nb) {
        float* f = S.fc + 6 * b;
        f[0] = a[h].x; f[1] = a[h].y; f[2] = a[h].z; f[3] = a[h].w; f[4] = c[h].x; f[5] = c[h].y;
      }
    }
    __syncwarp();
  }
  return lcg_jump(seed, total_draws);
}

}  // namespace og
