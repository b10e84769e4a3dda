// One-pass FP32 Conjugate Residual iteration for the inner solves of the
// mixed-precision pressure solve: the whole iteration of
// CONJUGATE_RESIDUAL::solvePCR (CONJUGATE_RESIDUAL.inl:139-160) in one
// TMA-staged z-marching kernel, 12 words per row of DRAM traffic instead of
// the 16 of the two-kernel split (pcr_phase_a + pressure_update_tma).
//
// Two changes make one pass possible:
//  * the preconditioner is folded into the stored vectors: t = s/diag and
//    q = Ap/diag are kept instead of s = A r and Ap, so the residual update
//    r -= alpha Ap/diag is r -= alpha q, and the search-direction update
//    Ap = s + beta Ap is q = t + beta q: no 1/diag at the halo;
//  * alpha of the next iteration needs (Ap, Ap/diag) of the next direction,
//    which expands exactly into inner products this pass can form at its
//    own cells:  (s + b Ap, (s + b Ap)/diag) = mu + 2 b nu + b^2 omega with
//    mu = (s', t'), nu = (s', q), omega = (Ap, q) (s' the new A r,
//    q the direction just used), so the four sums delta = (r', s'), mu, nu,
//    omega are reduced in one pass and alpha, beta both follow from them.
//
// Iteration k (state: r_k, t_k = s_k/diag, q_{k-1}, d_{k-1}, x_k; alpha_k,
// beta_k from the previous pass):
//   q_k = t_k + beta_k q_{k-1}     d_k = r_k + beta_k d_{k-1}
//   x  += alpha_k d_k               r_{k+1} = r_k - alpha_k q_k
//   s_{k+1} = J diag(m^-1) J^T r_{k+1},  t_{k+1} = s_{k+1}/diag
// with r_{k+1} formed at every halo cell from r, t, q (so r, t and q are
// read there and are double-buffered: pass k reads set (k & 1) and writes
// the other; x and d are read and written at own cells only, in place).
//
// The set-up pass (state `setup`, alpha = beta = 0, d = t = q = 0) forms
// s_0 = A r_0 and delta_0, mu_0 with the same kernel.
//
// Included by esf_solver.cu inside namespace esf after esf_tma.cuh (it reuses
// that kernel's tile geometry, mbarrier/TMA helpers and stencil stages).
#pragma once

struct FusedMaps {
  CUtensorMap r[2], t[2], q[2];  // box 72 x 10 at (x0 - 4, y0 - 1)
  CUtensorMap iv, x, d;          // box 64 x 8 at (x0, y0)
  CUtensorMap m;                 // padded node m^-1, box 68 x 9 at (x0, y0)
};
struct FusedPtrs {
  float* r[2];
  float* t[2];
  float* q[2];
  float* x;
  float* d;
};

constexpr int FU_OFF_R = 0, FU_OFF_T = TMA_HALO_SLOT, FU_OFF_Q = 2 * TMA_HALO_SLOT,
              FU_OFF_IV = 3 * TMA_HALO_SLOT, FU_OFF_X = FU_OFF_IV + TMA_OWN_BYTES,
              FU_OFF_D = FU_OFF_X + TMA_OWN_BYTES, FU_OFF_M = FU_OFF_D + TMA_OWN_BYTES;
constexpr int FU_STAGE_BYTES = FU_OFF_M + TMA_NODE_SLOT;  // 17536
static_assert(FU_OFF_IV % 128 == 0 && FU_OFF_X % 128 == 0 && FU_OFF_D % 128 == 0 &&
                  FU_OFF_M % 128 == 0 && FU_STAGE_BYTES % 128 == 0,
              "fused stage layout");
constexpr int FU_OFF_BAR = TMA_STAGES * FU_STAGE_BYTES;
constexpr int FU_OFF_P = FU_OFF_BAR + 128;
constexpr int FU_OFF_SQ = FU_OFF_P + TW_PP * HY * 4;
constexpr int FU_OFF_A = FU_OFF_SQ + TW_PP * HY * 4;
constexpr int FU_OFF_B = FU_OFF_A + TW_NP * NYN * 4;
constexpr int FU_OFF_C = FU_OFF_B + TW_NP * NYN * 4;
constexpr int FU_OFF_RED = (FU_OFF_C + TW_NP * NYN * 4 + 15) / 16 * 16;
constexpr int FU_SMEM = FU_OFF_RED + 32 * 8;  // about 47 KB: four blocks per SM
constexpr int FU_SUMS = 4;                    // delta, mu, nu, omega

// Scalars after a fused pass: totals of (r', s'), (s', t'), (s', q), (Ap, q).
__device__ __forceinline__ void finish_fused(PcrState* st, double dl, double mu, double nu,
                                             double om) {
  if (st->rebase) {
    // (double-float run) r was replaced by the FP64 residual (b - A x)/diag
    // and this pass kept q, d and e: the scalars of the pass that produced
    // the old r, recomputed for the new one
    const double beta = (st->deltaPrev > 0.0) ? dl / st->deltaPrev : 0.0;
    double den = mu + 2.0 * beta * nu + beta * beta * om;
    if (!(den > 0.0)) den = mu;
    st->beta = beta;
    st->alpha = (den > 0.0) ? dl / den : 0.0;
    st->delta = dl;
    st->delta0 = dl;
    st->rebase = 0;
    st->iter++;
    st->iter0 = st->iter;
    if (!(dl > 0.0)) {
      st->converged = 1;
      st->done = 1;
    }
  } else if (st->setup) {
    st->delta = dl;
    st->delta0 = dl;
    st->beta = 0.0;
    st->alpha = (mu > 0.0) ? dl / mu : 0.0;  // first direction is r: (Ap, Ap/diag) = mu
    st->setup = 0;
    st->iter0 = st->iter;
    if (!(dl > 0.0)) {  // zero right-hand side: nothing to do
      st->converged = 1;
      st->done = 1;
    }
  } else {
    const double beta = dl / st->delta;
    double den = mu + 2.0 * beta * nu + beta * beta * om;
    if (!(den > 0.0)) den = mu;  // rounding guard; (Ap, Ap/diag) is positive
    st->beta = beta;
    st->alpha = (den > 0.0) ? dl / den : 0.0;
    st->deltaPrev = st->delta;
    st->delta = dl;
    st->iter++;
    if (dl <= st->eps * st->eps * st->delta0 || (st->cap > 0 && st->iter - st->iter0 >= st->cap)) {
      st->converged = 1;
      st->done = 1;
    }
  }
  st->pp ^= 1;
  if (!(dl == dl) || !(mu == mu) || !(nu == nu) || !(om == om)) {
    st->status = ESF_ERR_NUMERIC;
    st->done = 1;
  }
}

// Double-float ("df") arithmetic on FP32 pairs (hi, lo), value hi + lo with
// |lo| <= ulp(hi)/2: a 48-bit significand from FP32 instructions only, by
// the error-free transformations of Knuth (TwoSum) and Dekker (the product
// error of an FMA). Explicit _rn intrinsics keep the compiler from
// contracting or reordering them.
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v)));
}
// y + a x (x df; y, a FP32)
__device__ __forceinline__ float2 df_axpy(float a, float2 x, float y) {
  const float ph = __fmul_rn(a, x.x);
  const float pl = __fmaf_rn(a, x.x, -ph);
  const float2 s = df_two_sum(y, ph);
  const float t = __fadd_rn(__fmaf_rn(a, x.y, pl), s.y);
  return df_two_sum(s.x, t);
}
// e + a d (e, d df; a FP32)
__device__ __forceinline__ float2 df_add_scaled(float2 e, float a, float2 d) {
  const float ph = __fmul_rn(a, d.x);
  const float pl = __fmaf_rn(a, d.x, -ph);
  const float2 s = df_two_sum(e.x, ph);
  const float t = __fadd_rn(__fadd_rn(__fmaf_rn(a, d.y, pl), e.y), s.y);
  return df_two_sum(s.x, t);
}

// One block's share of a pass: the 64 x 8-cell column (bx, by) over the cell
// layers bz*cz .. bz*cz+cz-1 of the scene (g, tm, p, partial, st), whose
// pass has nb blocks; bid is this block's place among them (the order in
// which the last block folds the partial sums).
//
// X64: the correction e (since the last FP64 check, which folds it into
// the FP64 solution) and the direction d are double-float pairs (edf, ddf:
// (hi, lo) per cell, interleaved) and move by plain 16-byte loads and
// stores of each thread's two cells, prefetched one layer ahead, instead of
// the TMA own-cell boxes; r, t, q and the stencil stay FP32. An FP32 iterate
// cannot hold the corrections of the operator's slowest modes: its rounding
// (relative 2^-24 per cell) reaches the residual amplified by up to kappa
// (about 5e7 at 256^3 cells), and an FP32 direction lets x and the recursive
// residual drift apart by as much. With both at a 48-bit significand one
// FP32 Krylov run reaches the FP64 tolerance in about the FP64 solver's
// iteration count, without the restarts of iterative refinement. (FP64
// arithmetic for the two updates kept the FP64 pipe 67% busy at half the
// DRAM bandwidth; the df updates are about 33 FP32 instructions a cell.)
// Both updates use the FP32 alpha and beta that update r and q.
template <bool X64>
__device__ __forceinline__ void fused_pass(const GridDev& g, const FusedMaps& tm, const FusedPtrs& p,
                                           float* edf, float* ddf, double* partial, PcrState* st,
                                           int cz, int bx, int by, int bz, int nb, int bid,
                                           unsigned char* smem) {
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem + FU_OFF_BAR);
  float* sP = reinterpret_cast<float*>(smem + FU_OFF_P);
  float* sQ = reinterpret_cast<float*>(smem + FU_OFF_SQ);
  float* sA = reinterpret_cast<float*>(smem + FU_OFF_A);
  float* sB = reinterpret_cast<float*>(smem + FU_OFF_B);
  float* sC = reinterpret_cast<float*>(smem + FU_OFF_C);
  double* sred = reinterpret_cast<double*>(smem + FU_OFF_RED);
  __shared__ bool amLast;
  if (st->done) return;
  if (st->iter >= st->maxIt) {
    if (bid == 0 && threadIdx.x == 0) st->done = 1;
    return;
  }
  const int pin = st->pp & 1, pout = pin ^ 1;
  // rebase pass (X64 only): alpha 0, q and d carried over unchanged
  const bool rb = X64 && st->rebase;
  const float alpha = rb ? 0.0f : (float)st->alpha, beta = (float)st->beta;
  const int tid = threadIdx.x;
  const int x0 = bx * TXW, y0 = by * TY, z0 = bz * cz;
  const int z1 = min(z0 + cz, g.cZ);
  const int nsteps = z1 - z0 + 2;  // cell layers z0-1 .. z1

  const CUtensorMap* mR = pin ? &tm.r[1] : &tm.r[0];
  const CUtensorMap* mT = pin ? &tm.t[1] : &tm.t[0];
  const CUtensorMap* mQ = pin ? &tm.q[1] : &tm.q[0];
  auto stage = [&](int i) { return smem + (i % TMA_STAGES) * FU_STAGE_BYTES; };
  auto issue = [&](int i) {
    const int kk = z0 - 1 + i;
    unsigned char* s = stage(i);
    unsigned long long* b = &bar[i % TMA_STAGES];
    const bool own = kk >= z0 && kk < z1;
    const bool node = kk >= z0;
    mbar_expect_tx(b, 3 * TMA_HALO_BYTES + (own ? (X64 ? 1 : 3) * TMA_OWN_BYTES : 0) +
                          (node ? TMA_NODE_BYTES : 0));
    tma_load_3d(s + FU_OFF_R, mR, x0 - 4, y0 - 1, kk, b);
    tma_load_3d(s + FU_OFF_T, mT, x0 - 4, y0 - 1, kk, b);
    tma_load_3d(s + FU_OFF_Q, mQ, x0 - 4, y0 - 1, kk, b);
    if (own) {
      tma_load_3d(s + FU_OFF_IV, &tm.iv, x0, y0, kk, b);
      if (!X64) {
        tma_load_3d(s + FU_OFF_X, &tm.x, x0, y0, kk, b);
        tma_load_3d(s + FU_OFF_D, &tm.d, x0, y0, kk, b);
      }
    }
    if (node) tma_load_3d(s + FU_OFF_M, &tm.m, x0, y0, kk, b);
  };
  if (tid == 0) {
    for (int i = 0; i < TMA_STAGES; i++) mbar_init(&bar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int i = 0; i < TMA_STAGES && i < nsteps; i++) issue(i);
  }
  __syncthreads();

  const int lane = tid & 31, w = tid >> 5;
  const int cx = 2 * lane;
  const int cgx = x0 + cx, cgy = y0 + w;
  const bool cin = cgx < g.cX && cgy < g.cY;  // cX is a multiple of 4
  const long long ccol = cgx + (long long)cgy * g.cX;
  const int bM = (cx + 4) + (w + 1) * TMA_HW;
  const int pM = (cx + 2) + (w + 1) * TW_PP;
  const int oM = cx + w * TXW;                  // own pair in the 64 x 8 boxes
  const int pN0 = (cx + 1) + w * TW_PP;
  const int mN = cx + w * TMA_NW;
  const int aN = cx + w * TW_NP;
  const bool hasE = tid < TW_RING;
  int eh = 0, ey = 0;
  if (tid < TW_HX) {
    eh = tid;
  } else if (tid < 2 * TW_HX) {
    eh = tid - TW_HX;
    ey = HY - 1;
  } else {
    const int e = tid - 2 * TW_HX;
    ey = 1 + (e >> 1);
    eh = (e & 1) ? TW_HX - 1 : 0;
  }
  const int bE = (eh + 3) + ey * TMA_HW, pE = (eh + 1) + ey * TW_PP;
  const bool hasN = tid < TW_NODE_EXTRA;
  const int enx = tid < TY ? TW_NX - 1 : tid - TY, eny = tid < TY ? tid : NYN - 1;
  const int pNE = (enx + 1) + eny * TW_PP, mNE = enx + eny * TMA_NW, aNE = enx + eny * TW_NP;

  // (selects, not indexing, keep the parameter structs out of local memory)
  float* rOut = pout ? p.r[1] : p.r[0];
  float* qOut = pout ? p.q[1] : p.q[0];
  float* tOut = pout ? p.t[1] : p.t[0];
  float sDl = 0, sMu = 0, sNu = 0, sOm = 0;
  float prev0 = 0, prev1 = 0, prevE = 0, vOwn0 = 0, vOwn1 = 0;
  float qCur0 = 0, qCur1 = 0, ivCur0 = 0, ivCur1 = 0;
  float mpx0 = 0, mpy0 = 0, mpz0 = 0, mpx1 = 0, mpy1 = 0, mpz1 = 0, mpxE = 0, mpyE = 0, mpzE = 0;
  float4 eNext = make_float4(0.f, 0.f, 0.f, 0.f), dNext = make_float4(0.f, 0.f, 0.f, 0.f);
  if (X64 && cin && z0 < z1) {
    const long long o = ccol + (long long)z0 * g.cslab;
    eNext = *reinterpret_cast<const float4*>(edf + 2 * o);
    dNext = *reinterpret_cast<const float4*>(ddf + 2 * o);
  }
  bool ok = true;
  int landed = 0;
  int issued = TMA_STAGES < nsteps ? TMA_STAGES : nsteps;
  for (int i = 0; i < nsteps; i++) {
    const int kk = z0 - 1 + i;
    if (ok) {
      ok = mbar_wait(&bar[i % TMA_STAGES], (unsigned)(i / TMA_STAGES) & 1u);
      if (ok) landed = i + 1;
    }
    const unsigned char* s = stage(i);
    const float* R = reinterpret_cast<const float*>(s + FU_OFF_R);
    const float* Tt = reinterpret_cast<const float*>(s + FU_OFF_T);
    const float* Qq = reinterpret_cast<const float*>(s + FU_OFF_Q);
    // this thread's cells of layer kk-1 (for the output in (c))
    const float qPrev0 = qCur0, qPrev1 = qCur1, ivPrev0 = ivCur0, ivPrev1 = ivCur1;
    // (a) r' = r - alpha (t + beta q) at the tile and halo cells of layer kk
    {
      const float2 r2 = *reinterpret_cast<const float2*>(R + bM);
      const float2 t2 = *reinterpret_cast<const float2*>(Tt + bM);
      const float2 q2 = *reinterpret_cast<const float2*>(Qq + bM);
      const float qn0 = rb ? q2.x : __fmaf_rn(beta, q2.x, t2.x), qn1 = rb ? q2.y : __fmaf_rn(beta, q2.y, t2.y);
      const float v0 = __fmaf_rn(-alpha, qn0, r2.x), v1 = __fmaf_rn(-alpha, qn1, r2.y);
      *reinterpret_cast<float2*>(sP + pM) = make_float2(prev0 + v0, prev1 + v1);
      *reinterpret_cast<float2*>(sQ + pM) = make_float2(prev0 - v0, prev1 - v1);
      vOwn0 = prev0;
      vOwn1 = prev1;
      prev0 = v0;
      prev1 = v1;
      if (kk >= z0 && kk < z1 && cin) {
        const float2 iv = *reinterpret_cast<const float2*>(s + FU_OFF_IV + 4 * oM);
        const long long o = ccol + (long long)kk * g.cslab;
        if constexpr (X64) {
          const float4 ev = eNext, dv = dNext;
          if (kk + 1 < z1) {  // the next layer's e and d, in flight during this one
            eNext = *reinterpret_cast<const float4*>(edf + 2 * (o + g.cslab));
            dNext = *reinterpret_cast<const float4*>(ddf + 2 * (o + g.cslab));
          }
          const float2 dn0 = rb ? make_float2(dv.x, dv.y) : df_axpy(beta, make_float2(dv.x, dv.y), r2.x);
          const float2 dn1 = rb ? make_float2(dv.z, dv.w) : df_axpy(beta, make_float2(dv.z, dv.w), r2.y);
          const float2 en0 = df_add_scaled(make_float2(ev.x, ev.y), alpha, dn0);
          const float2 en1 = df_add_scaled(make_float2(ev.z, ev.w), alpha, dn1);
          *reinterpret_cast<float4*>(ddf + 2 * o) = make_float4(dn0.x, dn0.y, dn1.x, dn1.y);
          *reinterpret_cast<float4*>(edf + 2 * o) = make_float4(en0.x, en0.y, en1.x, en1.y);
        } else {
          const float2 xv = *reinterpret_cast<const float2*>(s + FU_OFF_X + 4 * oM);
          const float2 dv = *reinterpret_cast<const float2*>(s + FU_OFF_D + 4 * oM);
          const float dn0 = __fmaf_rn(beta, dv.x, r2.x), dn1 = __fmaf_rn(beta, dv.y, r2.y);
          *reinterpret_cast<float2*>(p.d + o) = make_float2(dn0, dn1);
          *reinterpret_cast<float2*>(p.x + o) =
              make_float2(__fmaf_rn(alpha, dn0, xv.x), __fmaf_rn(alpha, dn1, xv.y));
        }
        *reinterpret_cast<float2*>(rOut + o) = make_float2(v0, v1);
        *reinterpret_cast<float2*>(qOut + o) = make_float2(qn0, qn1);
        // (Ap, q) = (q diag, q); an approximate quotient is plenty for a sum
        // that only sets the step length
        if (iv.x > 0.0f) sOm += __fdividef(qn0 * qn0, iv.x);
        if (iv.y > 0.0f) sOm += __fdividef(qn1 * qn1, iv.y);
        qCur0 = qn0;
        qCur1 = qn1;
        ivCur0 = iv.x;
        ivCur1 = iv.y;
      }
    }
    if (hasE) {
      const float v = __fmaf_rn(-alpha, __fmaf_rn(beta, Qq[bE], Tt[bE]), R[bE]);
      sP[pE] = prevE + v;
      sQ[pE] = prevE - v;
      prevE = v;
    }
    __syncthreads();
    // (b) node layer kk: J^T r' scaled by m^-1, paired with node layer kk-1
    if (kk >= z0) {
      const float* M = reinterpret_cast<const float*>(s + FU_OFF_M);
      {
        const float a0 = sP[pN0], b0 = sP[pN0 + TW_PP];
        const float2 a12 = *reinterpret_cast<const float2*>(sP + pN0 + 1);
        const float2 b12 = *reinterpret_cast<const float2*>(sP + pN0 + 1 + TW_PP);
        const float qa0 = sQ[pN0], qb0 = sQ[pN0 + TW_PP];
        const float2 qa12 = *reinterpret_cast<const float2*>(sQ + pN0 + 1);
        const float2 qb12 = *reinterpret_cast<const float2*>(sQ + pN0 + 1 + TW_PP);
        const float2 mi = *reinterpret_cast<const float2*>(M + mN);
        const float ab1 = a12.x + b12.x;
        const float mx0 = ((a0 + b0) - ab1) * mi.x;
        const float my0 = ((a0 + a12.x) - (b0 + b12.x)) * mi.x;
        const float mz0 = ((qa0 + qa12.x) + (qb0 + qb12.x)) * mi.x;
        const float mx1 = (ab1 - (a12.y + b12.y)) * mi.y;
        const float my1 = ((a12.x + a12.y) - (b12.x + b12.y)) * mi.y;
        const float mz1 = ((qa12.x + qa12.y) + (qb12.x + qb12.y)) * mi.y;
        if (kk >= z0 + 1) {
          *reinterpret_cast<float2*>(sA + aN) = make_float2(mpx0 + mx0, mpx1 + mx1);
          *reinterpret_cast<float2*>(sB + aN) = make_float2(mpy0 + my0, mpy1 + my1);
          *reinterpret_cast<float2*>(sC + aN) = make_float2(mz0 - mpz0, mz1 - mpz1);
        }
        mpx0 = mx0; mpy0 = my0; mpz0 = mz0;
        mpx1 = mx1; mpy1 = my1; mpz1 = mz1;
      }
      if (hasN) {
        const int s00 = pNE, s10 = s00 + 1, s01 = s00 + TW_PP, s11 = s01 + 1;
        const float mi = M[mNE];
        const float mx = ((sP[s00] + sP[s01]) - (sP[s10] + sP[s11])) * mi;
        const float my = ((sP[s00] + sP[s10]) - (sP[s01] + sP[s11])) * mi;
        const float mz = ((sQ[s00] + sQ[s10]) + (sQ[s01] + sQ[s11])) * mi;
        if (kk >= z0 + 1) {
          sA[aNE] = mpxE + mx;
          sB[aNE] = mpyE + my;
          sC[aNE] = mz - mpzE;
        }
        mpxE = mx; mpyE = my; mpzE = mz;
      }
    }
    __syncthreads();
    if (tid == 0 && ok && i + TMA_STAGES < nsteps) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(i + TMA_STAGES);
      issued = i + TMA_STAGES + 1;
    }
    // (c) s' and t' = s'/diag at the tile's cells of layer kk-1
    if (kk >= z0 + 1 && cin) {
      const float2 A01 = *reinterpret_cast<const float2*>(sA + aN);
      const float A2 = sA[aN + 2];
      const float2 B01 = *reinterpret_cast<const float2*>(sA + aN + TW_NP);
      const float B2 = sA[aN + 2 + TW_NP];
      const float2 c01 = *reinterpret_cast<const float2*>(sB + aN);
      const float c2 = sB[aN + 2];
      const float2 e01 = *reinterpret_cast<const float2*>(sB + aN + TW_NP);
      const float e2 = sB[aN + 2 + TW_NP];
      const float2 f01 = *reinterpret_cast<const float2*>(sC + aN);
      const float f2 = sC[aN + 2];
      const float2 g01 = *reinterpret_cast<const float2*>(sC + aN + TW_NP);
      const float g2 = sC[aN + 2 + TW_NP];
      const float mid = A01.y + B01.y;
      const float xp0 = mid - (A01.x + B01.x);
      const float yp0 = (e01.x + e01.y) - (c01.x + c01.y);
      const float zp0 = (f01.x + f01.y) + (g01.x + g01.y);
      const float xp1 = (A2 + B2) - mid;
      const float yp1 = (e01.y + e2) - (c01.y + c2);
      const float zp1 = (f01.y + f2) + (g01.y + g2);
      const float o0 = xp0 + yp0 + zp0, o1 = xp1 + yp1 + zp1;
      const float t0 = __fmul_rn(ivPrev0, o0), t1 = __fmul_rn(ivPrev1, o1);
      *reinterpret_cast<float2*>(tOut + ccol + (long long)(kk - 1) * g.cslab) = make_float2(t0, t1);
      sDl += vOwn0 * o0 + vOwn1 * o1;
      sMu += o0 * t0 + o1 * t1;
      sNu += o0 * qPrev0 + o1 * qPrev1;
    }
  }
  if (__syncthreads_or(!ok)) {
    if (tid == 0) {
      st->status = ESF_ERR_CUDA;
      st->done = 1;
      for (int j = landed; j < issued; j++)
        mbar_wait(&bar[j % TMA_STAGES], (unsigned)(j / TMA_STAGES) & 1u);
    }
    return;
  }
  // the four sums: block partials, folded in block order by the last block
  const double pDl = block_sum<NT>((double)sDl, sred);
  const double pMu = block_sum<NT>((double)sMu, sred);
  const double pNu = block_sum<NT>((double)sNu, sred);
  const double pOm = block_sum<NT>((double)sOm, sred);
  if (tid == 0) {
    partial[bid] = pDl;
    partial[nb + bid] = pMu;
    partial[2 * nb + bid] = pNu;
    partial[3 * nb + bid] = pOm;
    __threadfence();
    const unsigned t = atomicAdd(&st->ticket[1], 1u);
    amLast = (t + 1 == (unsigned)nb);
  }
  __syncthreads();
  if (!amLast) return;
  __threadfence();
  auto fold = [&](int h) {
    double a = 0;
    for (int q = tid; q < nb; q += NT) a += __ldcg(partial + h * nb + q);
    return block_sum<NT>(a, sred);
  };
  const double tDl = fold(0), tMu = fold(1), tNu = fold(2), tOm = fold(3);
  if (tid == 0) {
    st->ticket[1] = 0;
    finish_fused(st, tDl, tMu, tNu, tOm);
  }
}

__global__ void __launch_bounds__(NT, 4) pcr_iteration_fused(GridDev g, const __grid_constant__ FusedMaps tm,
                                                             FusedPtrs p, double* partial, PcrState* st,
                                                             int cz) {
  extern __shared__ __align__(128) unsigned char smem[];
  fused_pass<false>(g, tm, p, nullptr, nullptr, partial, st, cz, blockIdx.x, blockIdx.y, blockIdx.z,
                    gridDim.x * gridDim.y * gridDim.z,
                    blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z), smem);
}

// The same pass with the correction and direction in double-float
// (ESF_MIXED_X64).
__global__ void __launch_bounds__(NT, 4) pcr_iteration_fused_x64(GridDev g, const __grid_constant__ FusedMaps tm,
                                                                 FusedPtrs p, float* edf, float* ddf,
                                                                 double* partial, PcrState* st, int cz) {
  extern __shared__ __align__(128) unsigned char smem[];
  fused_pass<true>(g, tm, p, edf, ddf, partial, st, cz, blockIdx.x, blockIdx.y, blockIdx.z,
                   gridDim.x * gridDim.y * gridDim.z,
                   blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z), smem);
}

// ---- several scenes' inner solves in one launch (continuous batching).
// A task is one scene's inner solve: its grid, tensor maps, vectors, partial
// sums and state, and its pass's shape (cz layers per block, gx x gy x gz
// blocks). Tasks live in device memory (tensor maps there must be 64-byte
// aligned; the host writes them before the launches that read them).
struct FusedTask {
  FusedMaps tm;
  GridDev g;
  FusedPtrs p;
  double* partial;
  PcrState* st;
  int cz, gx, gy, gz;
};
static_assert(alignof(FusedTask) >= 64 && sizeof(FusedTask) % 64 == 0, "tensor maps need 64-byte alignment");
// The launch's list: entry k is (task slot, first block of that task in the
// launch); blocks [first_k, first_{k+1}) run task k's pass, so each task's
// blocks see the same (bx, by, bz), block count and block order as a launch
// of that scene alone, and their sums fold to the same bits.
constexpr int FU_MAX_BATCH = 256;
struct FusedBatch {
  int n;
  int slot[FU_MAX_BATCH];
  int first[FU_MAX_BATCH + 1];
};

__global__ void __launch_bounds__(NT, 4) pcr_iteration_fused_batch(const FusedTask* tasks,
                                                                   const __grid_constant__ FusedBatch b) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int blk = blockIdx.x;
  int lo = 0, hi = b.n - 1;  // the last k with first[k] <= blk
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (b.first[mid] <= blk) lo = mid;
    else hi = mid - 1;
  }
  const FusedTask& t = tasks[b.slot[lo]];
  const int local = blk - b.first[lo];
  const int nb = t.gx * t.gy * t.gz;
  if (local >= nb) return;
  const int bx = local % t.gx, by = (local / t.gx) % t.gy, bz = local / (t.gx * t.gy);
  fused_pass<false>(t.g, t.tm, t.p, nullptr, nullptr, t.partial, t.st, t.cz, bx, by, bz, nb, local, smem);
}

// The states of a batch's tasks, in list order, for one copy to the host.
__global__ void gather_task_states(const FusedTask* tasks, const __grid_constant__ FusedBatch b,
                                   PcrState* out) {
  for (int k = threadIdx.x; k < b.n; k += blockDim.x) out[k] = *tasks[b.slot[k]].st;
}
