// TMA-staged FP32 update kernel of the pressure PCR (the hot kernel of the
// mixed-precision inner solve): x += alpha d, v = r - alpha Ap/diag and
// s = J diag(m^-1) J^T v with the partial r.s, as pressure_stencil<float,
// S_UPDATE> computes them, with the inputs of each z-layer brought into
// shared memory by cp.async.bulk.tensor into a 2-deep ring of stages, so
// that each block has the next layer (~15 KB) in flight while it computes
// the current one, and four blocks fit per SM (a 3-deep ring fits three,
// and measured 6% slower at 256^3).
//
// Per layer and block (tile of 64 x 8 cells):
//   r, Ap, 1/diag : box 72 x 10 at (x0 - 4, y0 - 1)  (halo x0-1..x0+64 inside;
//                   x0 - 4 keeps the innermost coordinate 16-byte aligned)
//   x, d          : box 64 x 8 at (x0, y0), own layers only
//   m^-1 (nodes)  : box 68 x 9 at (x0, y0) of a node array padded to a row
//                   pitch that is a multiple of 4 floats, boundary and padding
//                   nodes zero
// Out-of-range boxes read zeros (TMA fill), which is the value the stencil
// gives cells and nodes outside the grid. The arithmetic is the same as the
// register kernel's, in the same order, so both give the same bits.
//
// Included by esf_solver.cu inside namespace esf, after the register kernel
// (it reuses its tile constants, upd_r and the block reductions).
#pragma once

struct TmaMaps {
  CUtensorMap r, ap, iv, x, d, m;
};

// Tile: 64 x 8 cells (TXW x TY), 256 threads; thread (lane, w) owns the
// cell pair (2 lane, 2 lane + 1) of row w, so neighbouring values come in
// 8-byte shared-memory loads and the pair shares its middle sums.
constexpr int TXW = 64;
constexpr int TW_HX = TXW + 2;   // halo columns x0-1 .. x0+64
constexpr int TW_PP = 68;        // sP/sQ row pitch; halo column h at index h + 1
constexpr int TW_NX = TXW + 1;   // node columns x0 .. x0+64
constexpr int TW_NP = 66;        // sA/sB/sC row pitch
constexpr int TMA_HW = 72, TMA_HH = 10;  // r/Ap/1/diag box: x0-4 .. x0+67, y0-1 .. y0+8
constexpr int TMA_NW = 68, TMA_NH = 9;   // m^-1 node box: x0 .. x0+67, y0 .. y0+8
constexpr int TMA_STAGES = 2;
// stage layout, each piece 128-byte aligned
constexpr int TMA_HALO_BYTES = TMA_HW * TMA_HH * 4;   // 2880
constexpr int TMA_HALO_SLOT = 2944;                   // 23 x 128
constexpr int TMA_OWN_BYTES = TXW * TY * 4;           // 2048
constexpr int TMA_NODE_BYTES = TMA_NW * TMA_NH * 4;   // 2448
constexpr int TMA_NODE_SLOT = 2560;                   // 20 x 128
constexpr int TMA_OFF_R = 0, TMA_OFF_AP = TMA_HALO_SLOT, TMA_OFF_IV = 2 * TMA_HALO_SLOT,
              TMA_OFF_X = 3 * TMA_HALO_SLOT, TMA_OFF_D = TMA_OFF_X + TMA_OWN_BYTES,
              TMA_OFF_M = TMA_OFF_D + TMA_OWN_BYTES;
constexpr int TMA_STAGE_BYTES = TMA_OFF_M + TMA_NODE_SLOT;  // 15488
static_assert(NT == 256 && TY == 8 && TX == 32, "thread (lane, w) owns a cell pair of row w");
static_assert(TMA_HALO_BYTES <= TMA_HALO_SLOT && TMA_NODE_BYTES <= TMA_NODE_SLOT &&
                  TMA_OFF_X % 128 == 0 && TMA_OFF_D % 128 == 0 && TMA_OFF_M % 128 == 0 &&
                  TMA_STAGE_BYTES % 128 == 0,
              "TMA stage layout");
// ring slots: the halo ring (rows y0-1 and y0+8, columns x0-1 and x0+64) and
// the last node column and row, one per thread
constexpr int TW_RING = 2 * TW_HX + 2 * TY;   // 148
constexpr int TW_NODE_EXTRA = TY + TW_NX;     // 73
// dynamic shared memory of the kernel
constexpr int TW_OFF_BAR = TMA_STAGES * TMA_STAGE_BYTES;
constexpr int TW_OFF_P = TW_OFF_BAR + 128;
constexpr int TW_OFF_Q = TW_OFF_P + TW_PP * HY * 4;
constexpr int TW_OFF_A = TW_OFF_Q + TW_PP * HY * 4;
constexpr int TW_OFF_B = TW_OFF_A + TW_NP * NYN * 4;
constexpr int TW_OFF_C = TW_OFF_B + TW_NP * NYN * 4;
constexpr int TW_OFF_RED = (TW_OFF_C + TW_NP * NYN * 4 + 15) / 16 * 16;
constexpr int TW_OFF_ACC = TW_OFF_RED + 32 * 8;
constexpr int TW_SMEM = TW_OFF_ACC + 2 * NT * 4;  // about 45 KB: four blocks per SM
// bounded waits: 2^18 polls before a block reports a stuck copy. An
// unsuccessful mbarrier.try_wait suspends the thread for its own time limit
// first (measured on GB300: ~3.8 us a poll), so the wait gives up after about
// one second, far beyond any copy that lands.
constexpr unsigned TMA_WAIT_LIMIT = 1u << 18;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// true once the phase with the given parity has completed; false after the
// poll limit
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  const unsigned a = smem_u32(bar);
  for (unsigned n = 0; n < TMA_WAIT_LIMIT; n++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Grid of the kernel: 64-cell tiles in x, the register kernel's tiles in y
// and z (same z-chunks), so that each block's r.s partials can be filed
// under the two 32-cell tiles of the register kernel's grid.
static inline dim3 tma_grid(const GridDev& g, int cz) {
  return dim3((g.cX + TXW - 1) / TXW, (g.cY + TY - 1) / TY, (g.cZ + cz - 1) / cz);
}

__global__ void __launch_bounds__(NT, 4) pressure_update_tma(GridDev g, const __grid_constant__ TmaMaps tm,
                                                             float* __restrict__ xout,
                                                             float* __restrict__ sout, double* partial,
                                                             PcrState* st, int cz) {
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem + TW_OFF_BAR);
  float* sP = reinterpret_cast<float*>(smem + TW_OFF_P);
  float* sQ = reinterpret_cast<float*>(smem + TW_OFF_Q);
  float* sA = reinterpret_cast<float*>(smem + TW_OFF_A);
  float* sB = reinterpret_cast<float*>(smem + TW_OFF_B);
  float* sC = reinterpret_cast<float*>(smem + TW_OFF_C);
  double* sred = reinterpret_cast<double*>(smem + TW_OFF_RED);
  float* sAcc = reinterpret_cast<float*>(smem + TW_OFF_ACC);
  __shared__ bool amLast;
  if (st->done) return;
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * TXW, y0 = blockIdx.y * TY, z0 = blockIdx.z * cz;
  const int z1 = min(z0 + cz, g.cZ);
  const float alpha = (float)st->alpha;
  const int nsteps = z1 - z0 + 2;  // cell layers z0-1 .. z1

  auto stage = [&](int i) { return smem + (i % TMA_STAGES) * TMA_STAGE_BYTES; };
  // the loads of step i (cell layer z0 - 1 + i) into stage i % TMA_STAGES
  auto issue = [&](int i) {
    const int kk = z0 - 1 + i;
    unsigned char* s = stage(i);
    unsigned long long* b = &bar[i % TMA_STAGES];
    const bool own = kk >= z0 && kk < z1;
    const bool node = kk >= z0;
    mbar_expect_tx(b, 3 * TMA_HALO_BYTES + (own ? 2 * TMA_OWN_BYTES : 0) + (node ? TMA_NODE_BYTES : 0));
    tma_load_3d(s + TMA_OFF_R, &tm.r, x0 - 4, y0 - 1, kk, b);
    tma_load_3d(s + TMA_OFF_AP, &tm.ap, x0 - 4, y0 - 1, kk, b);
    tma_load_3d(s + TMA_OFF_IV, &tm.iv, x0 - 4, y0 - 1, kk, b);
    if (own) {
      tma_load_3d(s + TMA_OFF_X, &tm.x, x0, y0, kk, b);
      tma_load_3d(s + TMA_OFF_D, &tm.d, x0, y0, kk, b);
    }
    if (node) tma_load_3d(s + TMA_OFF_M, &tm.m, x0, y0, kk, b);
  };
  if (tid == 0) {
    for (int i = 0; i < TMA_STAGES; i++) mbar_init(&bar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int i = 0; i < TMA_STAGES && i < nsteps; i++) issue(i);
  }
  __syncthreads();

  const int lane = tid & 31, w = tid >> 5;
  const int cx = 2 * lane;  // first cell of the pair, tile coordinates
  const int cgx = x0 + cx, cgy = y0 + w;
  // cX is a multiple of 4, so the pair is in or out of the grid together
  const bool cin = cgx < g.cX && cgy < g.cY;
  const long long ccol = cgx + (long long)cgy * g.cX;
  // main slots (even offsets: 8-byte aligned pairs)
  const int bM = (cx + 4) + (w + 1) * TMA_HW;   // halo columns cx+1, cx+2 in the box
  const int pM = (cx + 2) + (w + 1) * TW_PP;    // same in sP/sQ
  const int pN0 = (cx + 1) + w * TW_PP;         // node pair: halo column cx, row w
  const int mN = cx + w * TMA_NW;               // node pair in the m box
  const int aN = cx + w * TW_NP;                // node pair in sA/sB/sC
  // ring slots
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

  float acc0 = 0, acc1 = 0;
  float prev0 = 0, prev1 = 0, prevE = 0, vOwn0 = 0, vOwn1 = 0;
  float mpx0 = 0, mpy0 = 0, mpz0 = 0, mpx1 = 0, mpy1 = 0, mpz1 = 0, mpxE = 0, mpyE = 0, mpzE = 0;
  // A wait that times out leaves this thread computing on stale shared data
  // (every index is data-independent, so all accesses stay in bounds); the
  // block reports it once, after the loop.
  bool ok = true;
  int landed = 0;                                          // thread 0: steps < landed arrived
  int issued = TMA_STAGES < nsteps ? TMA_STAGES : nsteps;  // thread 0: steps < issued issued
  for (int i = 0; i < nsteps; i++) {
    const int kk = z0 - 1 + i;
    if (ok) {
      ok = mbar_wait(&bar[i % TMA_STAGES], (unsigned)(i / TMA_STAGES) & 1u);
      if (ok) landed = i + 1;
    }
    const unsigned char* s = stage(i);
    const float* R = reinterpret_cast<const float*>(s + TMA_OFF_R);
    const float* AP = reinterpret_cast<const float*>(s + TMA_OFF_AP);
    const float* IV = reinterpret_cast<const float*>(s + TMA_OFF_IV);
    // (a) stencil input of cell layer kk: P = v(k-1) + v(k), Q = v(k-1) - v(k)
    {
      const float2 r2 = *reinterpret_cast<const float2*>(R + bM);
      const float2 a2 = *reinterpret_cast<const float2*>(AP + bM);
      const float2 i2 = *reinterpret_cast<const float2*>(IV + bM);
      const float v0 = upd_r(r2.x, alpha, a2.x, i2.x), v1 = upd_r(r2.y, alpha, a2.y, i2.y);
      *reinterpret_cast<float2*>(sP + pM) = make_float2(prev0 + v0, prev1 + v1);
      *reinterpret_cast<float2*>(sQ + pM) = make_float2(prev0 - v0, prev1 - v1);
      vOwn0 = prev0;  // this thread's cells in layer kk-1, for r.s in (c)
      vOwn1 = prev1;
      prev0 = v0;
      prev1 = v1;
    }
    if (hasE) {
      const float v = upd_r(R[bE], alpha, AP[bE], IV[bE]);
      sP[pE] = prevE + v;
      sQ[pE] = prevE - v;
      prevE = v;
    }
    // x += alpha d on the tile's own cells
    if (kk >= z0 && kk < z1 && cin) {
      const float2 xv = *reinterpret_cast<const float2*>(s + TMA_OFF_X + 4 * (cx + w * TXW));
      const float2 dv = *reinterpret_cast<const float2*>(s + TMA_OFF_D + 4 * (cx + w * TXW));
      *reinterpret_cast<float2*>(xout + ccol + (long long)kk * g.cslab) =
          make_float2(xv.x + alpha * dv.x, xv.y + alpha * dv.y);
    }
    __syncthreads();
    // (b) node layer kk: J^T v scaled by m^-1, paired with node layer kk-1
    if (kk >= z0) {
      const float* M = reinterpret_cast<const float*>(s + TMA_OFF_M);
      {
        // halo columns cx, cx+1, cx+2 of rows w (a*) and w+1 (b*)
        const float a0 = sP[pN0], b0 = sP[pN0 + TW_PP];
        const float2 a12 = *reinterpret_cast<const float2*>(sP + pN0 + 1);
        const float2 b12 = *reinterpret_cast<const float2*>(sP + pN0 + 1 + TW_PP);
        const float qa0 = sQ[pN0], qb0 = sQ[pN0 + TW_PP];
        const float2 qa12 = *reinterpret_cast<const float2*>(sQ + pN0 + 1);
        const float2 qb12 = *reinterpret_cast<const float2*>(sQ + pN0 + 1 + TW_PP);
        const float2 mi = *reinterpret_cast<const float2*>(M + mN);
        const float ab1 = a12.x + b12.x;  // shared by both nodes' x differences
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
    // stage i is consumed: refill it with step i + TMA_STAGES
    if (tid == 0 && ok && i + TMA_STAGES < nsteps) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(i + TMA_STAGES);
      issued = i + TMA_STAGES + 1;
    }
    // (c) output cell layer kk-1: node columns cx, cx+1, cx+2 of rows w, w+1
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
      const float mid = A01.y + B01.y;  // shared by both cells' x differences
      const float xp0 = mid - (A01.x + B01.x);
      const float yp0 = (e01.x + e01.y) - (c01.x + c01.y);
      const float zp0 = (f01.x + f01.y) + (g01.x + g01.y);
      const float xp1 = (A2 + B2) - mid;
      const float yp1 = (e01.y + e2) - (c01.y + c2);
      const float zp1 = (f01.y + f2) + (g01.y + g2);
      const float o0 = xp0 + yp0 + zp0, o1 = xp1 + yp1 + zp1;
      *reinterpret_cast<float2*>(sout + ccol + (long long)(kk - 1) * g.cslab) = make_float2(o0, o1);
      acc0 += vOwn0 * o0;
      acc1 += vOwn1 * o1;
    }
  }
  if (__syncthreads_or(!ok)) {
    // a copy did not complete in time: report it, and wait (bounded) for the
    // copies still in flight before the block's shared memory is released
    if (tid == 0) {
      st->status = ESF_ERR_CUDA;
      st->done = 1;
      for (int j = landed; j < issued; j++)
        mbar_wait(&bar[j % TMA_STAGES], (unsigned)(j / TMA_STAGES) & 1u);
    }
    return;
  }
  // r.s: file the per-cell sums under the two 32-cell tiles of the register
  // kernel's grid and reduce each exactly as that kernel does (same thread
  // layout, same tree, same block order), so both kernels give the same bits
  {
    const int half = cx >> 5, ol = cx & 31;
    sAcc[half * NT + w * 32 + ol] = acc0;
    sAcc[half * NT + w * 32 + ol + 1] = acc1;
  }
  const int gxo = (g.cX + TX - 1) / TX;
  const int nOld = gxo * gridDim.y * gridDim.z;
  double part[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    __syncthreads();
    part[h] = block_sum<NT>((double)sAcc[h * NT + tid], sred);
  }
  if (tid == 0) {
    unsigned cnt = 0;
    for (int h = 0; h < 2; h++) {
      const int bxo = 2 * blockIdx.x + h;
      if (bxo < gxo) {
        partial[bxo + gxo * (blockIdx.y + gridDim.y * blockIdx.z)] = part[h];
        cnt++;
      }
    }
    __threadfence();
    const unsigned t = atomicAdd(&st->ticket[1], cnt);
    amLast = (t + cnt == (unsigned)nOld);
  }
  __syncthreads();
  if (!amLast) return;
  __threadfence();
  double a = 0;
  for (int q = tid; q < nOld; q += NT) a += __ldcg(partial + q);
  const double total = block_sum<NT>(a, sred);
  if (tid == 0) {
    st->ticket[1] = 0;
    finish_update(st, total);
  }
}
