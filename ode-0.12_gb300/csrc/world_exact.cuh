// world_exact.cuh -- dWorldStep (ode/src/step.cpp:187-846) for one world, one
// warp: islands as for QuickStep, then per island the joints ordered
// unbounded / mixed / LCP by the reference's two-ended scheme, the dense
// A = J invM J' + cfm / h, and the Dantzig LCP of ode/src/lcp.cpp with ODE's
// pivoting rules (index sets C and N, row / column swaps through row
// pointers, LDL' updates by rank-2 modification). Every lane runs the solver's
// control flow; vector loops and dot products are spread over the lanes.
//
// Scratch per world (global memory, X.off[w] floats into X.base): A and L
// (cap x cap, cap = the world's row capacity), 13 vectors of cap floats,
// JinvM (12 per row), 9 int vectors of cap, and 12 floats per body.
#pragma once
#include "world_solve.cuh"

namespace og {

struct ExactDev {
  float* base;
  const long long* off;    // [n_worlds] float offset of each world's scratch
  const int* cap;          // [n_worlds] rows the scratch holds
};

OG_D float xw_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
OG_D float xw_dot(const float* a, const float* b, int n, int lane) {
  float s = 0.f;
  for (int k = lane; k < n; k += 32) s += a[k] * b[k];
  return xw_sum(s);
}

// L x = b in place (unit lower triangular, rows of L at stride ns), in
// blocks of 32 rows with lane j owning row r0 + j: each lane first takes the
// dot product of its row with the solved part x[0, r0) (its own row, no
// reduction), then the block's triangle is solved through shuffles.
OG_D void xw_solve_l1(const float* L, float* B, int n, int ns, int lane) {
  for (int r0 = 0; r0 < n; r0 += 32) {
    const int r = r0 + lane;
    const int nbk = min(32, n - r0);
    float v = 0.f;
    if (r < n) {
      const float* Lr = L + (size_t)r * ns;
      float s = 0.f;
      for (int c = 0; c < r0; ++c) s += Lr[c] * B[c];
      v = B[r] - s;
    }
    for (int j = 0; j < nbk; ++j) {
      const float xj = __shfl_sync(kFull, v, j);
      if (lane > j && r < n) v -= L[(size_t)r * ns + r0 + j] * xj;
    }
    if (r < n) B[r] = v;
    __syncwarp();
  }
}
// L' x = b in place, blocks of 32 from the bottom; lane j owns row lo + j and
// reads column-wise across the lanes (rows of L are contiguous).
OG_D void xw_solve_l1t(const float* L, float* B, int n, int ns, int lane) {
  for (int hi = n; hi > 0; hi -= 32) {
    const int lo = max(0, hi - 32);
    const int a = lo + lane;
    float v = 0.f;
    if (a < hi) {
      float s = 0.f;
      for (int c = hi; c < n; ++c) s += L[(size_t)c * ns + a] * B[c];
      v = B[a] - s;
    }
    for (int j = hi - 1 - lo; j >= 0; --j) {
      const float xc = __shfl_sync(kFull, v, j);
      if (lane < j && a < hi) v -= L[(size_t)(lo + j) * ns + a] * xc;
    }
    if (a < hi) B[a] = v;
    __syncwarp();
  }
}
// A = L D L' in place (L below the diagonal), d = 1 / D
OG_D void xw_factor_ldlt(float* A, float* d, int n, int ns, int lane) {
  for (int i = 0; i < n; ++i) {
    float* ri = A + (size_t)i * ns;
    xw_solve_l1(A, ri, i, ns, lane);
    float s = 0.f;
    for (int j = lane; j < i; j += 32) {
      const float z = ri[j], l = z * d[j];
      ri[j] = l;
      s += z * l;
    }
    s = xw_sum(s);
    __syncwarp();
    if (lane == 0) d[i] = 1.0f / (ri[i] - s);
    __syncwarp();
  }
}
OG_D void xw_solve_ldlt(const float* L, const float* d, float* b, int n, int ns, int lane) {
  xw_solve_l1(L, b, n, ns, lane);
  for (int i = lane; i < n; i += 32) b[i] *= d[i];
  __syncwarp();
  xw_solve_l1t(L, b, n, ns, lane);
}

// _dLDLTAddTL (ode/src/matrix.cpp:260-336)
OG_D void xw_ldlt_add_tl(float* L, float* d, const float* a, int n, int ns, float* W1, float* W2, int lane) {
  if (n < 2) return;
  for (int j = lane; j < n; j += 32) {
    const float v = (j == 0) ? 0.f : a[j] * kSqrt1_2;
    W1[j] = v;
    W2[j] = v;
  }
  __syncwarp();
  const float W11 = (0.5f * a[0] + 1.f) * kSqrt1_2, W21 = (0.5f * a[0] - 1.f) * kSqrt1_2;
  float alpha1 = 1.f, alpha2 = 1.f;
  {
    float dee = d[0];
    float an = alpha1 + (W11 * W11) * dee;
    dee /= an;
    const float g1 = W11 * dee;
    dee *= alpha1;
    alpha1 = an;
    an = alpha2 - (W21 * W21) * dee;
    alpha2 = an;
    const float k1 = 1.f - W21 * g1, k2 = W21 * g1 * W11 - W21;
    for (int p = 1 + lane; p < n; p += 32) {
      const float Wp = W1[p], ell = L[(size_t)p * ns];
      W1[p] = Wp - W11 * ell;
      W2[p] = k1 * Wp + k2 * ell;
    }
  }
  __syncwarp();
  for (int j = 1; j < n; ++j) {
    const float k1 = W1[j], k2 = W2[j];
    float dee = d[j];
    float an = alpha1 + (k1 * k1) * dee;
    dee /= an;
    const float g1 = k1 * dee;
    dee *= alpha1;
    alpha1 = an;
    an = alpha2 - (k2 * k2) * dee;
    dee /= an;
    const float g2 = k2 * dee;
    dee *= alpha2;
    alpha2 = an;
    __syncwarp();
    if (lane == 0) d[j] = dee;
    for (int p = j + 1 + lane; p < n; p += 32) {
      float* l = &L[(size_t)p * ns + j];
      float ell = *l;
      float Wp = W1[p] - k1 * ell;
      ell += g1 * Wp;
      W1[p] = Wp;
      Wp = W2[p] - k2 * ell;
      ell -= g2 * Wp;
      W2[p] = Wp;
      *l = ell;
    }
    __syncwarp();
  }
}

// shift v[from..from+count) to v[from-1..) (memmove left by one)
template <class T>
OG_D void xw_shift_left(T* v, int from, int count, int lane) {
  for (int base = 0; base < count; base += 32) {
    const int k = base + lane;
    T val{};
    if (k < count) val = v[from + k];
    __syncwarp();
    if (k < count) v[from + k - 1] = val;
    __syncwarp();
  }
}

// _dRemoveRowCol (ode/src/matrix.cpp:402-434)
OG_D void xw_remove_row_col(float* A, int n, int ns, int r, int lane) {
  if (r >= n - 1) return;
  if (r > 0) {
    for (int i = 0; i < r; ++i) xw_shift_left(A + (size_t)i * ns, r + 1, n - r - 1, lane);
    for (int i = r; i < n - 1; ++i) {
      for (int k = lane; k < r; k += 32) A[(size_t)i * ns + k] = A[(size_t)(i + 1) * ns + k];
      __syncwarp();
    }
  }
  for (int i = r; i < n - 1; ++i) {
    for (int k = lane; k < n - r - 1; k += 32) A[(size_t)i * ns + r + k] = A[(size_t)(i + 1) * ns + r + 1 + k];
    __syncwarp();
  }
}

// The LCP problem of one island (lcp.cpp's dLCP with row pointers).
struct XLcp {
  int n, ns, nub, nC, nN;
  float* Ab;          // A data, n rows of ns
  int* rowp;          // row offsets into Ab
  float *x, *b, *w, *lo, *hi, *L, *d, *Dell, *ell, *tmp, *dx, *W1, *W2, *t;
  int *state, *findex, *p, *C;
  OG_D float* A(int i) const { return Ab + rowp[i]; }
  OG_D float geta(int i, int j) const { return (i > j) ? A(i)[j] : A(j)[i]; }
};

// swapRowsAndCols + swapProblem (lcp.cpp:148-267)
OG_D void xw_swap_problem(XLcp& S, int i1, int i2, bool fast, int lane) {
  if (i1 == i2) return;
  float* A_i1 = S.A(i1);
  float* A_i2 = S.A(i2);
  for (int i = i1 + 1 + lane; i < i2; i += 32) {
    float* A_i_i1 = S.A(i) + i1;
    A_i1[i] = *A_i_i1;
    *A_i_i1 = A_i2[i];
  }
  __syncwarp();
  if (lane == 0) {
    A_i1[i2] = A_i1[i1];
    A_i1[i1] = A_i2[i1];
    A_i2[i1] = A_i2[i2];
    if (fast) { const int t = S.rowp[i1]; S.rowp[i1] = S.rowp[i2]; S.rowp[i2] = t; }
  }
  __syncwarp();
  if (!fast)
    for (int k = lane; k <= i2; k += 32) { const float t = A_i1[k]; A_i1[k] = A_i2[k]; A_i2[k] = t; }
  for (int j = i2 + 1 + lane; j < S.n; j += 32) {
    float* A_j = S.A(j);
    const float t = A_j[i1]; A_j[i1] = A_j[i2]; A_j[i2] = t;
  }
  if (lane == 0) {
#define XSW(v) { const auto t_ = S.v[i1]; S.v[i1] = S.v[i2]; S.v[i2] = t_; }
    XSW(x) XSW(b) XSW(w) XSW(lo) XSW(hi) XSW(p) XSW(state) XSW(findex)
#undef XSW
  }
  __syncwarp();
}

OG_D void xw_gather_dell(XLcp& S, int i, int lane) {
  const float* aptr = S.A(i);
  for (int j = lane; j < S.nC; j += 32) S.Dell[j] = (j < S.nub) ? aptr[j] : aptr[S.C[j]];
  __syncwarp();
}

OG_D void xw_transfer_i_to_C(XLcp& S, int i, int lane) {
  if (S.nC > 0) {
    float* Lt = S.L + (size_t)S.nC * S.ns;
    for (int j = lane; j < S.nC; j += 32) Lt[j] = S.ell[j];
    const float dd = S.A(i)[i] - xw_dot(S.ell, S.Dell, S.nC, lane);
    __syncwarp();
    if (lane == 0) S.d[S.nC] = 1.0f / dd;
  } else if (lane == 0) {
    S.d[0] = 1.0f / S.A(i)[i];
  }
  __syncwarp();
  xw_swap_problem(S, S.nC, i, true, lane);
  if (lane == 0) S.C[S.nC] = S.nC;
  __syncwarp();
  S.nC++;
}

OG_D void xw_transfer_i_from_N_to_C(XLcp& S, int i, int lane) {
  if (S.nC > 0) {
    xw_gather_dell(S, i, lane);
    xw_solve_l1(S.L, S.Dell, S.nC, S.ns, lane);
    float* Lt = S.L + (size_t)S.nC * S.ns;
    for (int j = lane; j < S.nC; j += 32) Lt[j] = S.ell[j] = S.Dell[j] * S.d[j];
    __syncwarp();
    const float dd = S.A(i)[i] - xw_dot(S.ell, S.Dell, S.nC, lane);
    __syncwarp();
    if (lane == 0) S.d[S.nC] = 1.0f / dd;
  } else if (lane == 0) {
    S.d[0] = 1.0f / S.A(i)[i];
  }
  __syncwarp();
  xw_swap_problem(S, S.nC, i, true, lane);
  if (lane == 0) S.C[S.nC] = S.nC;
  __syncwarp();
  S.nN--;
  S.nC++;
}

// _dLDLTRemove (ode/src/matrix.cpp:348-399) with p = C
OG_D void xw_ldlt_remove(XLcp& S, int n2, int r, int lane) {
  if (r == n2 - 1) return;
  const int* p = S.C;
  if (r == 0) {
    float* a = S.t;
    const int p0 = p[0];
    for (int i = lane; i < n2; i += 32) a[i] = -S.geta(p[i], p0) + (i == 0 ? 1.0f : 0.f);
    __syncwarp();
    xw_ldlt_add_tl(S.L, S.d, a, n2, S.ns, S.W1, S.W2, lane);
  } else {
    float* t = S.t;
    const float* Lr = S.L + (size_t)r * S.ns;
    for (int i = lane; i < r; i += 32) t[i] = Lr[i] / S.d[i];
    __syncwarp();
    float* a = t + r;
    const int p_r = p[r];
    for (int i = lane; i < n2 - r; i += 32) {
      const float* Li = S.L + (size_t)(r + i) * S.ns;
      float s = 0.f;
      for (int k = 0; k < r; ++k) s += Li[k] * t[k];
      a[i] = s - S.geta(p[r + i], p_r) + (i == 0 ? 1.0f : 0.f);
    }
    __syncwarp();
    xw_ldlt_add_tl(S.L + (size_t)r * S.ns + r, S.d + r, a, n2 - r, S.ns, S.W1, S.W2, lane);
  }
  xw_remove_row_col(S.L, n2, S.ns, r, lane);
  xw_shift_left(S.d, r + 1, n2 - r - 1, lane);
}

OG_D void xw_transfer_i_from_C_to_N(XLcp& S, int i, int lane) {
  const int nC = S.nC;
  int j = 0, last_idx = -1;
  for (; j < nC; ++j) {   // every lane scans (C is read-only here)
    if (S.C[j] == nC - 1) last_idx = j;
    if (S.C[j] == i) break;
  }
  __syncwarp();
  if (j < nC) {
    xw_ldlt_remove(S, nC, j, lane);
    int k = last_idx;
    if (k == -1)
      for (k = j + 1; k < nC; ++k)
        if (S.C[k] == nC - 1) break;
    __syncwarp();
    if (lane == 0 && k < nC) S.C[k] = S.C[j];
    __syncwarp();
    xw_shift_left(S.C, j + 1, nC - j - 1, lane);
  }
  xw_swap_problem(S, i, nC - 1, true, lane);
  S.nN++;
  S.nC = nC - 1;
}

// solve1 (lcp.cpp:704-757)
OG_D void xw_solve1(XLcp& S, float* a, int i, int dir, bool only_transfer, int lane) {
  if (S.nC <= 0) return;
  xw_gather_dell(S, i, lane);
  xw_solve_l1(S.L, S.Dell, S.nC, S.ns, lane);
  for (int j = lane; j < S.nC; j += 32) S.ell[j] = S.Dell[j] * S.d[j];
  __syncwarp();
  if (!only_transfer) {
    for (int j = lane; j < S.nC; j += 32) S.tmp[j] = S.ell[j];
    __syncwarp();
    xw_solve_l1t(S.L, S.tmp, S.nC, S.ns, lane);
    for (int j = lane; j < S.nC; j += 32) a[S.C[j]] = dir > 0 ? -S.tmp[j] : S.tmp[j];
    __syncwarp();
  }
}

// dSolveLCP (lcp.cpp:784-1073). A rows at rowp (identity on entry), lower
// triangle used. Returns true when the solver stopped on s <= 0.
OG_D bool xw_solve_lcp(XLcp& S, int lane) {
  const int n = S.n;
  if (S.nub >= n) {
    xw_factor_ldlt(S.Ab, S.d, n, S.ns, lane);
    xw_solve_ldlt(S.Ab, S.d, S.b, n, S.ns, lane);
    for (int k = lane; k < n; k += 32) S.x[k] = S.b[k];
    __syncwarp();
    return false;
  }
  float* dw = S.tmp;   // delta_w shares tmp (lcp.cpp:835-836)
  for (int k = lane; k < n; k += 32) { S.x[k] = 0.f; S.p[k] = k; S.state[k] = 0; S.w[k] = 0.f; }
  __syncwarp();
  for (int k = S.nub; k < n; ++k) {
    if (S.findex[k] >= 0) continue;
    if (S.lo[k] == -INFINITY && S.hi[k] == INFINITY) {
      xw_swap_problem(S, S.nub, k, false, lane);
      S.nub++;
    }
  }
  S.nC = 0;
  S.nN = 0;
  if (S.nub > 0) {
    for (int j = 0; j < S.nub; ++j) {
      const float* Aj = S.A(j);
      float* Lj = S.L + (size_t)j * S.ns;
      for (int c = lane; c <= j; c += 32) Lj[c] = Aj[c];
    }
    __syncwarp();
    xw_factor_ldlt(S.L, S.d, S.nub, S.ns, lane);
    for (int k = lane; k < S.nub; k += 32) S.x[k] = S.b[k];
    __syncwarp();
    xw_solve_ldlt(S.L, S.d, S.x, S.nub, S.ns, lane);
    for (int k = lane; k < S.nub; k += 32) { S.w[k] = 0.f; S.C[k] = k; }
    __syncwarp();
    S.nC = S.nub;
  }
  {
    int at_end = 0;
    for (int k = n - 1; k >= S.nub; k--)
      if (S.findex[k] >= 0) {
        xw_swap_problem(S, k, n - 1 - at_end, true, lane);
        at_end++;
      }
  }
  const int adj_nub = S.nub;
  bool hit_first_friction = false, err = false;
  for (int i = adj_nub; i < n && !err; ++i) {
    if (!hit_first_friction && S.findex[i] >= 0) {
      for (int j = lane; j < n; j += 32) dw[S.p[j]] = S.x[j];
      __syncwarp();
      for (int k = i + lane; k < n; k += 32) {
        const float wfk = dw[S.findex[k]];
        if (wfk == 0.f) { S.hi[k] = 0.f; S.lo[k] = 0.f; }
        else { S.hi[k] = fabsf(S.hi[k] * wfk); S.lo[k] = -S.hi[k]; }
      }
      __syncwarp();
      hit_first_friction = true;
    }
    const float wi = xw_dot(S.A(i), S.x, S.nC, lane) + xw_dot(S.A(i) + S.nC, S.x + S.nC, S.nN, lane) - S.b[i];
    __syncwarp();
    if (lane == 0) S.w[i] = wi;
    __syncwarp();
    if (S.lo[i] == 0.f && wi >= 0.f) {
      S.nN++;
      if (lane == 0) S.state[i] = 0;
    } else if (S.hi[i] == 0.f && wi <= 0.f) {
      S.nN++;
      if (lane == 0) S.state[i] = 1;
    } else if (wi == 0.f) {
      xw_solve1(S, S.dx, i, 0, true, lane);
      xw_transfer_i_to_C(S, i, lane);
    } else {
      for (int guard = 0; guard < 4 * n + 8; ++guard) {
        const float wi_ = S.w[i];
        const int dir = (wi_ <= 0.f) ? 1 : -1;
        const float dirf = (float)dir;
        xw_solve1(S, S.dx, i, dir, false, lane);
        {
          const int nC = S.nC, nN = S.nN;
          const float* ai = S.A(i);
          for (int k = lane; k < nN; k += 32) {
            const float* Ak = S.A(k + nC);
            float s = 0.f;
            for (int c = 0; c < nC; ++c) s += Ak[c] * S.dx[c];
            dw[nC + k] = dir > 0 ? s + ai[nC + k] : s - ai[nC + k];
          }
        }
        const float dwi = xw_dot(S.A(i), S.dx, S.nC, lane) + S.A(i)[i] * dirf;
        __syncwarp();
        if (lane == 0) dw[i] = dwi;
        __syncwarp();
        // largest step: the first candidate (in the reference's scan order)
        // with the smallest step size
        int cmd = 1, si = 0;
        float s = -wi_ / dwi;
        if (dir > 0) {
          if (S.hi[i] < INFINITY) {
            const float s2 = (S.hi[i] - S.x[i]) * dirf;
            if (s2 < s) { s = s2; cmd = 3; }
          }
        } else {
          if (S.lo[i] > -INFINITY) {
            const float s2 = (S.lo[i] - S.x[i]) * dirf;
            if (s2 < s) { s = s2; cmd = 2; }
          }
        }
        float bv = INFINITY;
        int bpos = 0x7fffffff;
        for (int k = lane; k < S.nN; k += 32) {
          const int ik = S.nC + k;
          const float dk = dw[ik];
          if (!S.state[ik] ? dk < 0.f : dk > 0.f) {
            if (S.lo[ik] == 0.f && S.hi[ik] == 0.f) continue;
            const float s2 = -S.w[ik] / dk;
            if (s2 < bv || (s2 == bv && k < bpos)) { bv = s2; bpos = k; }
          }
        }
        for (int k = adj_nub + lane; k < S.nC; k += 32) {
          const float xk = S.dx[k];
          const int pos = S.nN + 2 * (k - adj_nub);
          if (xk < 0.f && S.lo[k] > -INFINITY) {
            const float s2 = (S.lo[k] - S.x[k]) / xk;
            if (s2 < bv || (s2 == bv && pos < bpos)) { bv = s2; bpos = pos; }
          }
          if (xk > 0.f && S.hi[k] < INFINITY) {
            const float s2 = (S.hi[k] - S.x[k]) / xk;
            if (s2 < bv || (s2 == bv && pos + 1 < bpos)) { bv = s2; bpos = pos + 1; }
          }
        }
        for (int o = 16; o > 0; o >>= 1) {
          const float ov = __shfl_xor_sync(kFull, bv, o);
          const int op = __shfl_xor_sync(kFull, bpos, o);
          if (ov < bv || (ov == bv && op < bpos)) { bv = ov; bpos = op; }
        }
        if (bpos != 0x7fffffff && bv < s) {
          s = bv;
          if (bpos < S.nN) { cmd = 4; si = S.nC + bpos; }
          else {
            const int q = bpos - S.nN;
            si = adj_nub + (q >> 1);
            cmd = (q & 1) ? 6 : 5;
          }
        }
        if (s <= 0.f) {   // the reference gives up here too (lcp.cpp:985-993)
          for (int k = i + lane; k < n; k += 32) { S.x[k] = 0.f; S.w[k] = 0.f; }
          __syncwarp();
          err = true;
          break;
        }
        for (int k = lane; k < S.nC; k += 32) S.x[k] += s * S.dx[k];
        for (int k = lane; k < S.nN; k += 32) S.w[S.nC + k] += s * dw[S.nC + k];
        __syncwarp();
        if (lane == 0) { S.x[i] += s * dirf; S.w[i] += s * dw[i]; }
        __syncwarp();
        switch (cmd) {
          case 1:
            if (lane == 0) S.w[i] = 0.f;
            __syncwarp();
            xw_transfer_i_to_C(S, i, lane);
            break;
          case 2:
            if (lane == 0) { S.x[i] = S.lo[i]; S.state[i] = 0; }
            S.nN++;
            break;
          case 3:
            if (lane == 0) { S.x[i] = S.hi[i]; S.state[i] = 1; }
            S.nN++;
            break;
          case 4:
            if (lane == 0) S.w[si] = 0.f;
            __syncwarp();
            xw_transfer_i_from_N_to_C(S, si, lane);
            break;
          case 5:
            if (lane == 0) { S.x[si] = S.lo[si]; S.state[si] = 0; }
            __syncwarp();
            xw_transfer_i_from_C_to_N(S, si, lane);
            break;
          default:
            if (lane == 0) { S.x[si] = S.hi[si]; S.state[si] = 1; }
            __syncwarp();
            xw_transfer_i_from_C_to_N(S, si, lane);
            break;
        }
        __syncwarp();
        if (cmd <= 3) break;
        if (guard == 4 * n + 7) err = true;   // bounded: a cycling pivot sequence ends the solve
      }
    }
  }
  // unpermute x and w (lcp.cpp:759-781)
  for (int j = lane; j < n; j += 32) S.tmp[j] = S.x[j];
  __syncwarp();
  for (int j = lane; j < n; j += 32) S.x[S.p[j]] = S.tmp[j];
  __syncwarp();
  for (int j = lane; j < n; j += 32) S.tmp[j] = S.w[j];
  __syncwarp();
  for (int j = lane; j < n; j += 32) S.w[S.p[j]] = S.tmp[j];
  __syncwarp();
  return err;
}

// info->nub of each joint's getInfo1 (ball.cpp:52, hinge.cpp:56,
// hinge2.cpp:84, slider.cpp:118, universal.cpp:267, fixed.cpp:54,
// amotor.cpp:194, contact.cpp:51-70)
OG_D int joint_nub(const BatchDev& d, const WorldDesc& D, int ord) {
  if (ord >= D.njp) {
    const DevSurface& S = d.surfaces[d.contacts[D.contact_off + ord - D.njp].surface];
    int nub = 0;
    if (S.mode & ODEGPU_CONTACT_MU2) {
      if (S.mu == INFINITY) nub++;
      if (S.mu2 == INFINITY) nub++;
    } else if (S.mu == INFINITY) {
      nub += 2;
    }
    return nub;
  }
  switch (d.joints[D.joint_off + ord].type) {
    case J_BALL: return 3;
    case J_HINGE: return 5;
    case J_HINGE2: return 4;
    case J_SLIDER: return 5;
    case J_UNIVERSAL: return 4;
    case J_FIXED: return 6;
    default: return 0;
  }
}

// Per-world scratch carve-up.
struct XWorld {
  float *A, *L, *x, *b, *w, *lo, *hi, *d, *Dell, *ell, *tmp, *dx, *W1, *W2, *t, *JinvM, *cforce, *tmp1;
  int *p, *C, *state, *findex, *rowp, *rq, *jm, *jnub, *jofs;
  float* jerp;
  int* seq;   // 2 * cap + 2 entries: the two-ended joint order
};
OG_D XWorld carve_exact(float* base, int cap) {
  XWorld X;
  float* f = base;
  const size_t cc = (size_t)cap * cap;
  X.A = f; f += cc;
  X.L = f; f += cc;
  X.x = f; f += cap; X.b = f; f += cap; X.w = f; f += cap; X.lo = f; f += cap; X.hi = f; f += cap;
  X.d = f; f += cap; X.Dell = f; f += cap; X.ell = f; f += cap; X.tmp = f; f += cap; X.dx = f; f += cap;
  X.W1 = f; f += cap; X.W2 = f; f += cap; X.t = f; f += cap;
  X.JinvM = f; f += (size_t)12 * cap;
  X.jerp = f; f += cap;
  X.cforce = f; f += 6 * kMaxB;
  X.tmp1 = f; f += 6 * kMaxB;
  int* ip = reinterpret_cast<int*>(f);
  X.p = ip; ip += cap; X.C = ip; ip += cap; X.state = ip; ip += cap; X.findex = ip; ip += cap;
  X.rowp = ip; ip += cap; X.rq = ip; ip += cap; X.jm = ip; ip += cap; X.jnub = ip; ip += cap;
  X.jofs = ip; ip += cap;
  X.seq = ip;
  return X;
}
// floats of scratch a world with `cap` rows needs
OG_HD constexpr long long exact_scratch_floats(int cap) {
  return 2LL * cap * cap + 40LL * cap + 12LL * kMaxB + 16;
}

// The regions of a dWorldStep: every world's row bound for this step (at
// most 3 rows per contact and 6 per persistent joint, within its row
// capacity; it also bounds the joint count, nj <= rows) and the float
// offsets of the worlds' regions, with their total. One block; each thread
// sums a run of worlds, then a block scan over the runs.
constexpr int kExactSizeThreads = 1024;
__global__ void __launch_bounds__(kExactSizeThreads)
exact_size_kernel(BatchDev d, int* cap, long long* off, long long* total) {
  __shared__ long long part[kExactSizeThreads];
  const int n = d.n_worlds, t = threadIdx.x;
  const int per = (n + kExactSizeThreads - 1) / kExactSizeThreads;
  const int w0 = min(n, t * per), w1 = min(n, w0 + per);
  long long sum = 0;
  for (int w = w0; w < w1; ++w) {
    const WorldDesc D = d.world[w];
    const long long bound = 6LL * D.njp + 3LL * d.ncontacts[w];
    const int c = (int)max(1LL, min(bound, (long long)min(D.row_cap, kMaxR)));
    cap[w] = c;
    sum += (exact_scratch_floats(c) + 3) & ~3LL;
  }
  part[t] = sum;
  __syncthreads();
  for (int o = 1; o < kExactSizeThreads; o <<= 1) {
    const long long v = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  long long base = part[t] - sum;
  for (int w = w0; w < w1; ++w) {
    off[w] = base;
    base += (exact_scratch_floats(cap[w]) + 3) & ~3LL;
  }
  if (t == kExactSizeThreads - 1) *total = part[t];
}

// The two-ended joint order of step.cpp:265-403 over island-local joints
// 0..nj-1 with (jm, jnub); returns the count of joints kept (m > 0) and their
// order in out[], and *nubj = the number of purely unbounded joints (which
// the reference hands to the LCP as its nub). a: 2 nj + 2 ints.
OG_D int exact_joint_order(const int* jm, const int* jnub, int nj, int* a, int* out, int* nubj) {
  int unb_start = nj, mix_start = nj, mix_end = nj, lcp_end = nj;
  int cur = lcp_end, src = 0;
  for (;;) {
    bool fwd_end = false;
    {
      int mixend = mix_end;
      for (;;) {
        if (src == nj) { lcp_end = cur; fwd_end = true; break; }
        const int k = src++;
        const int m = jm[k], nub = jnub[k];
        if (m <= 0) continue;
        if (nub == 0) {
          a[cur++] = k;
        } else if (nub < m) {
          if (unb_start == mix_start) {
            unb_start = mix_start = mix_start - 1;
            a[mix_start] = k;
          } else if (mixend != cur) {
            a[cur] = a[mixend];
            a[mixend] = k;
            ++mixend; ++cur;
          } else {
            a[cur] = k;
            mixend = cur = cur + 1;
          }
        } else {
          unb_start = unb_start - 1;
          a[unb_start] = k;
          lcp_end = cur;
          mix_end = mixend;
          cur = unb_start - 1;
          break;
        }
      }
    }
    if (fwd_end) break;
    bool bkw_end = false;
    {
      int mixstart = mix_start - 1;
      for (;;) {
        if (src == nj) { unb_start = cur + 1; mix_start = mixstart + 1; bkw_end = true; break; }
        const int k = src++;
        const int m = jm[k], nub = jnub[k];
        if (m <= 0) continue;
        if (nub == m) {
          a[cur--] = k;
        } else if (nub > 0) {
          if (mix_end == lcp_end) {
            const int e = mix_end;
            lcp_end = mix_end = mix_end + 1;
            a[e] = k;
          } else if (mixstart != cur) {
            a[cur] = a[mixstart];
            a[mixstart] = k;
            --mixstart; --cur;
          } else {
            a[cur] = k;
            mixstart = cur = cur - 1;
          }
        } else {
          const int e = lcp_end;
          lcp_end = lcp_end + 1;
          a[e] = k;
          unb_start = cur + 1;
          mix_start = mixstart + 1;
          cur = e + 1;
          break;
        }
      }
    }
    if (bkw_end) break;
  }
  *nubj = mix_start - unb_start;
  const int n = lcp_end - unb_start;
  for (int q = 0; q < n; ++q) out[q] = a[unb_start + q];
  return n;
}

// dxStepBody position / orientation update after the velocity update of
// step.cpp:790-806 (cf: J' lambda of the body, 6 floats)
OG_D bool integrate_exact_body(const BatchDev& d, const WorldDesc& D, int gb, const float* cf) {
  const float h = D.dt;
  float4 lv = d.lvel[gb], av = d.avel[gb];
  const float4 f = d.facc[gb], tq = d.tacc[gb];
  const float hm = h * d.invMass[gb];
  lv.x += (cf[0] + f.x) * hm; lv.y += (cf[1] + f.y) * hm; lv.z += (cf[2] + f.z) * hm;
  const float data[3] = {(cf[3] + tq.x) * h, (cf[4] + tq.y) * h, (cf[5] + tq.z) * h};
  float r3[3];
  mul0_331(r3, d.invIw + 12 * gb, data);
  av.x += r3[0]; av.y += r3[1]; av.z += r3[2];
  return step_body(d, gb, h, lv, av);
}

OG_D float dot6(const float* u, const float* v) {
  return u[0] * v[0] + u[1] * v[1] + u[2] * v[2] + u[3] * v[3] + u[4] * v[4] + u[5] * v[5];
}

// One dWorldStep of world w (after the collide kernel's controls, contacts and
// body prologue).
OG_D void world_exact(const BatchDev& d, const ExactDev& XD, int w, int step, const WarpSmem& S, int lane,
                      const StepOptions& opt) {
  const WorldDesc D = d.world[w];
  const int nc = d.ncontacts[w];
  const int cap = XD.cap[w];
  XWorld X = carve_exact(XD.base + XD.off[w], cap);
  for (int k = lane; k < 6 * D.nb; k += 32) X.cforce[k] = 0.f;
  int M = 0, nisl = 0;
  bool bad = false, nonfinite = false;
  if (D.njp + nc > kMaxR || D.njp + nc > cap) {
    if (lane == 0) atomicOr(&d.status[w], ST_TOO_LARGE);
  } else {
    const int nj = phase_islands(d, D, w, opt.host_adjacency ? 0 : nc, D.njp + nc, S, lane, &nisl);
    (void)nj;
    const float* stops = step_stops(d, D, step);
    const int jl_off = D.joint_off + D.contact_off;
    const float h1 = 1.0f / D.dt;
    const int* istart = d.island_jstart + D.body_off + w;
    for (int isl = 0; isl < nisl && !bad; ++isl) {
      const int js = istart[isl], je = istart[isl + 1], njl = je - js;
      // getInfo1 of the island's joints, in island order
      for (int k = lane; k < njl; k += 32) {
        const int ord = d.jlist[jl_off + js + k] & 0x3fffffff;
        int m;
        if (ord < D.njp) {
          const DevJoint& J = d.joints[D.joint_off + ord];
          const DevLimot lm1 = step_limot1(J, stops, ord);
          BodyRef B1, B2;
          load_body_ref(d, D.body_off + J.b1, B1);
          if (J.b2 >= 0) load_body_ref(d, D.body_off + J.b2, B2);
          m = persistent_info1(J, lm1, B1, J.b2 >= 0 ? &B2 : nullptr).m;
        } else {
          m = contact_info1(d.surfaces[d.contacts[D.contact_off + ord - D.njp].surface]);
        }
        X.jm[k] = m;
        X.jnub[k] = joint_nub(d, D, ord);
      }
      __syncwarp();
      int njr = 0, nubj = 0, m = 0;
      if (lane == 0) {
        // order, row offsets and the erp each joint sees (ball / fixed
        // joints leave theirs in the shared Info2 block, ball.cpp:59)
        njr = exact_joint_order(X.jm, X.jnub, njl, X.seq, X.rq, &nubj);
        float erp = D.erp;
        for (int q = 0; q < njr; ++q) {
          const int k = X.rq[q];
          const int ord = d.jlist[jl_off + js + k] & 0x3fffffff;
          X.jofs[q] = m;
          X.jerp[q] = erp;
          m += X.jm[k];
          if (ord < D.njp) {
            const DevJoint& J = d.joints[D.joint_off + ord];
            if (J.type == J_BALL || J.type == J_FIXED) erp = J.erp;
          }
        }
      }
      njr = __shfl_sync(kFull, njr, 0);
      nubj = __shfl_sync(kFull, nubj, 0);
      m = __shfl_sync(kFull, m, 0);
      __syncwarp();
      if (M + m > D.row_cap || m > cap) {
        if (lane == 0) atomicOr(&d.status[w], ST_ROW_OVERFLOW);
        bad = true;
        break;
      }
      if (m == 0) continue;
      // getInfo2 in the new order into the world's row store
      for (int q = lane; q < njr; q += 32) {
        const int k = X.rq[q];
        const int ord = d.jlist[jl_off + js + k] & 0x3fffffff;
        assemble_joint_rows(d, D, ord, M + X.jofs[q], X.jm[k], X.jerp[q], stops, nullptr);
      }
      __syncwarp();
      const float* rows = d.rows + (size_t)(D.row_off + M) * kRowWords;
      // per row: joint position, LCP bounds, J invM
      for (int q = lane; q < njr; q += 32) {
        const int mk = X.jm[X.rq[q]];
        for (int r = 0; r < mk; ++r) X.tmp[X.jofs[q] + r] = __int_as_float(q);
      }
      __syncwarp();
      for (int a = lane; a < m; a += 32) {
        const float* row = rows + (size_t)a * kRowWords;
        const int* ri = reinterpret_cast<const int*>(row);
        X.C[a] = __float_as_int(X.tmp[a]);   // joint position of row a (C is free until the LCP)
        X.lo[a] = row[kRowLo];
        X.hi[a] = row[kRowHi];
        const int fi = ri[kRowFindex];
        X.findex[a] = (fi == -1) ? -1 : fi - M;
        for (int half = 0; half < 2; ++half) {
          const int bt = ri[half ? kRowB2 : kRowB1];
          float* t = X.JinvM + (size_t)a * 12 + 6 * half;
          if (bt < 0) { for (int q = 0; q < 6; ++q) t[q] = 0.f; continue; }
          const int gb = D.body_off + bt;
          const float im = d.invMass[gb];
          const float* s = row + 6 * half;
          const float* iI = d.invIw + 12 * gb;
          for (int q = 0; q < 3; ++q) t[q] = s[q] * im;
          for (int q = 0; q < 3; ++q) t[3 + q] = s[3] * iI[q] + s[4] * iI[4 + q] + s[5] * iI[8 + q];
        }
      }
      __syncwarp();
      // A = J invM J' (lower triangle and diagonal blocks) + cfm / h; rhs
      for (int a = lane; a < m; a += 32) {
        const float* ra = rows + (size_t)a * kRowWords;
        const int* ria = reinterpret_cast<const int*>(ra);
        const int qa = X.C[a];
        const int end = X.jofs[qa] + X.jm[X.rq[qa]];
        const int ba[2] = {ria[kRowB1], ria[kRowB2]};
        const float* u = X.JinvM + (size_t)a * 12;
        float* Arow = X.A + (size_t)a * cap;
        // only joints sharing a body with row a's joint give non-zero blocks
        for (int c = 0; c < end; ++c) Arow[c] = 0.f;
        for (int q = 0; q <= qa; ++q) {
          const int ofs = X.jofs[q], mk = X.jm[X.rq[q]];
          const int* riq = reinterpret_cast<const int*>(rows + (size_t)ofs * kRowWords);
          const int qb1 = riq[kRowB1], qb2 = riq[kRowB2];
          if (q == qa) {
            for (int r = 0; r < mk; ++r) {
              const float* rc = rows + (size_t)(ofs + r) * kRowWords;
              float v = dot6(u, rc);
              if (ba[1] >= 0) v += dot6(u + 6, rc + 6);
              Arow[ofs + r] = v;
            }
            continue;
          }
          for (int half = 0; half < 2; ++half) {
            const int bt = ba[half];
            if (bt < 0) continue;
            const int oh = (qb1 == bt) ? 0 : (qb2 == bt ? 1 : -1);
            if (oh < 0) continue;
            for (int r = 0; r < mk; ++r)
              Arow[ofs + r] += dot6(u + 6 * half, rows + (size_t)(ofs + r) * kRowWords + 6 * oh);
          }
        }
        Arow[a] += ra[kRowCfm] * h1;
        float t1[6];
        float bb = ra[kRowC] * h1;
        body_tmp1(d, D.body_off + ba[0], h1, t1);
        bb -= dot6(ra, t1);
        if (ba[1] >= 0) {
          body_tmp1(d, D.body_off + ba[1], h1, t1);
          bb -= dot6(ra + 6, t1);
        }
        X.b[a] = bb;
        X.rowp[a] = a * cap;
      }
      __syncwarp();
      XLcp L;
      L.n = m; L.ns = cap; L.nub = nubj; L.nC = 0; L.nN = 0;
      L.Ab = X.A; L.rowp = X.rowp;
      L.x = X.x; L.b = X.b; L.w = X.w; L.lo = X.lo; L.hi = X.hi; L.L = X.L; L.d = X.d;
      L.Dell = X.Dell; L.ell = X.ell; L.tmp = X.tmp; L.dx = X.dx; L.W1 = X.W1; L.W2 = X.W2; L.t = X.t;
      L.state = X.state; L.findex = X.findex; L.p = X.p; L.C = X.C;
      const bool lcp_err = xw_solve_lcp(L, lane);
      if (lcp_err && lane == 0) atomicOr(&d.status[w], ST_LCP_STOP);
      // cforce = J' lambda, per joint in order (step.cpp:720-786); joint feedback
      for (int q = 0; q < njr; ++q) {
        const int ofs = X.jofs[q], mk = X.jm[X.rq[q]];
        const int* ri0 = reinterpret_cast<const int*>(rows + (size_t)ofs * kRowWords);
        const int ord = ri0[kRowJoint];
        float* fb = nullptr;   // dJointFeedback f1 t1 f2 t2 of the joint, when asked for
        if (ord < D.njp) { if (opt.feedback) fb = opt.feedback + (size_t)(D.joint_off + ord) * 12; }
        else if (opt.contact_feedback) fb = opt.contact_feedback + (size_t)(D.contact_off + ord - D.njp) * 12;
        for (int half = 0; half < 2; ++half) {
          const int bt = ri0[half ? kRowB2 : kRowB1];
          if (bt < 0) {
            if (lane < 6 && fb) fb[6 + lane] = 0.f;
            continue;
          }
          if (lane < 6) {
            float s = 0.f;
            for (int r = 0; r < mk; ++r) s += rows[(size_t)(ofs + r) * kRowWords + 6 * half + lane] * X.x[ofs + r];
            X.cforce[6 * bt + lane] += s;
            if (fb) fb[6 * half + lane] = s;
          }
          __syncwarp();
        }
      }
      M += m;
    }
  }
  __syncwarp();
  for (int b = lane; b < D.nb; b += 32) nonfinite |= integrate_exact_body(d, D, D.body_off + b, X.cforce + 6 * b);
  if (__any_sync(kFull, nonfinite) && lane == 0) atomicOr(&d.status[w], ST_NONFINITE);
  if (lane == 0) {
    d.nrows[w] = M;
    d.nislands[w] = nisl;
  }
  __syncwarp();
}

}  // namespace og
