// TMA-staged FP32 update kernel of the pressure PCR (the hot kernel of the
// mixed-precision inner solve): x += alpha d, v = r - alpha Ap/diag and
// s = J diag(m^-1) J^T v with the partial r.s, as pressure_stencil<float,
// S_UPDATE> computes them, with the inputs of each z-layer brought into
// shared memory by cp.async.bulk.tensor into a 4-deep ring of stages, so
// that each block keeps three layers (~25 KB) of loads in flight while it
// computes the current one instead of one layer of register prefetch.
//
// Per layer and block (tile of TX x TY cells):
//   r, Ap, 1/diag : box 40 x 10 at (x0 - 4, y0 - 1)  (halo x0-1..x0+32 inside;
//                   x0 - 4 keeps the innermost coordinate 16-byte aligned)
//   x, d          : box 32 x 8 at (x0, y0), own layers only
//   m^-1 (nodes)  : box 36 x 9 at (x0, y0) of a node array padded to a row
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

constexpr int TMA_HW = 40, TMA_HH = 10;  // halo box
constexpr int TMA_NW = 36, TMA_NH = 9;   // node box
constexpr int TMA_STAGES = 4;
// stage layout, each piece 128-byte aligned
constexpr int TMA_HALO_BYTES = TMA_HW * TMA_HH * 4;   // 1600
constexpr int TMA_HALO_SLOT = 1664;                   // 13 x 128
constexpr int TMA_OWN_BYTES = TX * TY * 4;            // 1024
constexpr int TMA_NODE_BYTES = TMA_NW * TMA_NH * 4;   // 1296
constexpr int TMA_NODE_SLOT = 1408;                   // 11 x 128
constexpr int TMA_OFF_R = 0, TMA_OFF_AP = TMA_HALO_SLOT, TMA_OFF_IV = 2 * TMA_HALO_SLOT,
              TMA_OFF_X = 3 * TMA_HALO_SLOT, TMA_OFF_D = TMA_OFF_X + TMA_OWN_BYTES,
              TMA_OFF_M = TMA_OFF_D + TMA_OWN_BYTES;
constexpr int TMA_STAGE_BYTES = TMA_OFF_M + TMA_NODE_SLOT;  // 8448
static_assert(TX == 32 && NT == TX * TY && NHALO - NT == 2 * HX + 2 * TY && NNODE - NT == NXN + TY,
              "row-aligned slots: warp w owns cell row w");
static_assert(TMA_HALO_BYTES <= TMA_HALO_SLOT && TMA_NODE_BYTES <= TMA_NODE_SLOT &&
                  TMA_OFF_X % 128 == 0 && TMA_OFF_D % 128 == 0 && TMA_OFF_M % 128 == 0 &&
                  TMA_STAGE_BYTES % 128 == 0,
              "TMA stage layout");
// bounded waits: ~2^24 polls (seconds) before a block reports a stuck copy
constexpr unsigned TMA_WAIT_LIMIT = 1u << 24;

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

__global__ void __launch_bounds__(NT) pressure_update_tma(GridDev g, const __grid_constant__ TmaMaps tm,
                                                          float* __restrict__ xout,
                                                          float* __restrict__ sout, double* partial,
                                                          PcrState* st, int cz) {
  __shared__ __align__(128) unsigned char stage[TMA_STAGES][TMA_STAGE_BYTES];
  __shared__ __align__(8) unsigned long long bar[TMA_STAGES];
  __shared__ float sP[NHALO], sQ[NHALO];
  __shared__ float sA[NNODE], sB[NNODE], sC[NNODE];
  __shared__ double sred[32];
  if (st->done) return;
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * cz;
  const int z1 = min(z0 + cz, g.cZ);
  const float alpha = (float)st->alpha;
  const int nsteps = z1 - z0 + 2;  // cell layers z0-1 .. z1

  // the loads of step i (cell layer z0 - 1 + i) into stage i % TMA_STAGES
  auto issue = [&](int i) {
    const int kk = z0 - 1 + i;
    unsigned char* s = stage[i % TMA_STAGES];
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

  // Slots are row-aligned so that a warp's shared-memory accesses are
  // contiguous (no bank conflicts): warp w owns cell row w, whose halo cells
  // are the interior halo row w+1 and whose nodes are node row w; the halo
  // ring (84 cells) and the last node row and column (41 nodes) go to the
  // first threads as a second slot.
  const int lane = tid & 31, w = tid >> 5;
  const int ccx = lane, ccy = w;
  const int cgx = x0 + ccx, cgy = y0 + ccy;
  const bool cin = cgx < g.cX && cgy < g.cY;
  const long long ccol = cgx + (long long)cgy * g.cX;
  const int hM = (lane + 1) + (w + 1) * HX, bM = (lane + 4) + (w + 1) * TMA_HW;
  const bool hasE = tid < NHALO - NT;
  int ehx = 0, ehy = 0;
  if (tid < HX) {
    ehx = tid;
  } else if (tid < 2 * HX) {
    ehx = tid - HX;
    ehy = HY - 1;
  } else {
    const int e = tid - 2 * HX;
    ehy = 1 + (e >> 1);
    ehx = (e & 1) ? HX - 1 : 0;
  }
  const int hE = ehx + ehy * HX, bE = (ehx + 3) + ehy * TMA_HW;
  const int nM = lane + w * NXN, sM = lane + w * HX, mM = lane + w * TMA_NW;
  const bool hasN = tid < NNODE - NT;
  const int enx = tid < NXN ? tid : NXN - 1, eny = tid < NXN ? NYN - 1 : tid - NXN;
  const int nE = enx + eny * NXN, sE = enx + eny * HX, mE = enx + eny * TMA_NW;
  float accT = 0;
  float prevM = 0, prevE = 0, vOwn = 0;
  float mpxM = 0, mpyM = 0, mpzM = 0, mpxE = 0, mpyE = 0, mpzE = 0;
  // A wait that times out leaves this thread computing on stale shared data
  // (every index is data-independent, so all accesses stay in bounds); the
  // block reports it once, after the loop, instead of paying a block-wide
  // vote per layer.
  bool ok = true;
  int landed = 0;                                          // thread 0: steps < landed arrived
  int issued = TMA_STAGES < nsteps ? TMA_STAGES : nsteps;  // thread 0: steps < issued issued
  for (int i = 0; i < nsteps; i++) {
    const int kk = z0 - 1 + i;
    if (ok) {
      ok = mbar_wait(&bar[i % TMA_STAGES], (unsigned)(i / TMA_STAGES) & 1u);
      if (ok) landed = i + 1;
    }
    const unsigned char* s = stage[i % TMA_STAGES];
    const float* R = reinterpret_cast<const float*>(s + TMA_OFF_R);
    const float* AP = reinterpret_cast<const float*>(s + TMA_OFF_AP);
    const float* IV = reinterpret_cast<const float*>(s + TMA_OFF_IV);
    // (a) stencil input of cell layer kk: P = v(k-1) + v(k), Q = v(k-1) - v(k)
    {
      const float v = upd_r(R[bM], alpha, AP[bM], IV[bM]);
      sP[hM] = prevM + v;
      sQ[hM] = prevM - v;
      vOwn = prevM;  // v of this thread's cell in layer kk-1, for r.s in (c)
      prevM = v;
    }
    if (hasE) {
      const float v = upd_r(R[bE], alpha, AP[bE], IV[bE]);
      sP[hE] = prevE + v;
      sQ[hE] = prevE - v;
      prevE = v;
    }
    // x += alpha d on the tile's own cells
    if (kk >= z0 && kk < z1 && cin) {
      const float* X = reinterpret_cast<const float*>(s + TMA_OFF_X);
      const float* D = reinterpret_cast<const float*>(s + TMA_OFF_D);
      const float xv = X[tid], dv = D[tid];
      xout[ccol + (long long)kk * g.cslab] = xv + alpha * dv;
    }
    __syncthreads();
    // (b) node layer kk: J^T v scaled by m^-1, paired with node layer kk-1
    if (kk >= z0) {
      const float* M = reinterpret_cast<const float*>(s + TMA_OFF_M);
      auto node = [&](int ns, int s00, int mi_at, float& mpx, float& mpy, float& mpz) {
        const int s10 = s00 + 1, s01 = s00 + HX, s11 = s01 + 1;
        const float mi = M[mi_at];
        const float mx = ((sP[s00] + sP[s01]) - (sP[s10] + sP[s11])) * mi;
        const float my = ((sP[s00] + sP[s10]) - (sP[s01] + sP[s11])) * mi;
        const float mz = ((sQ[s00] + sQ[s10]) + (sQ[s01] + sQ[s11])) * mi;
        if (kk >= z0 + 1) {
          sA[ns] = mpx + mx;
          sB[ns] = mpy + my;
          sC[ns] = mz - mpz;
        }
        mpx = mx;
        mpy = my;
        mpz = mz;
      };
      node(nM, sM, mM, mpxM, mpyM, mpzM);
      if (hasN) node(nE, sE, mE, mpxE, mpyE, mpzE);
    }
    __syncthreads();
    // stage i is consumed: refill it with step i + TMA_STAGES
    if (tid == 0 && ok && i + TMA_STAGES < nsteps) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(i + TMA_STAGES);
      issued = i + TMA_STAGES + 1;
    }
    // (c) output cell layer kk-1
    if (kk >= z0 + 1 && cin) {
      const int n00 = ccx + ccy * NXN, n10 = n00 + 1, n01 = n00 + NXN, n11 = n01 + 1;
      const float xp = (sA[n10] + sA[n11]) - (sA[n00] + sA[n01]);
      const float yp = (sB[n01] + sB[n11]) - (sB[n00] + sB[n10]);
      const float zp = (sC[n00] + sC[n10]) + (sC[n01] + sC[n11]);
      const float o = xp + yp + zp;
      sout[ccol + (long long)(kk - 1) * g.cslab] = o;
      accT += vOwn * o;
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
  const double bs = block_sum<NT>((double)accT, sred);
  const int nblocks = gridDim.x * gridDim.y * gridDim.z;
  double total;
  if (last_block_sum<NT>(bs, partial, &st->ticket[1], nblocks, &total, sred) && threadIdx.x == 0)
    finish_update(st, total);
}
