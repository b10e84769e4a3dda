// Two-level preconditioner of the mixed-precision inner pressure solves.
//
// Jacobi-preconditioned Conjugate Residual needs thousands of iterations on
// J M^-1 J^T because of a family of slow modes: the cell grid's sign
// patterns (-1)^x, (-1)^y, ..., (-1)^(x+y+z) times slowly varying envelopes,
// which J^T maps to (nearly) zero (the spurious pressure modes of the
// trilinear-velocity / constant-pressure pair). The coarse space Z holds the
// 8 sign patterns on each block of bs^3 cells (bs a multiple of 32), K =
// 8 x blocks columns, and the inner solves use
//     M^-1 = D^-1 + Z F Z^T,   F = (Z^T A Z + eps max(diag) I)^-1
// (an additive two-level preconditioner: symmetric positive definite, one
// operator product per iteration). The regularisation keeps F bounded on
// the coarse space's null directions (patterns whose envelope J^T annihilates).
//
// In the one-pass iteration the preconditioner acts where t = M^-1 s is
// read: the stored t is the Jacobi part s/diag, and the pass adds (Z c)(cell)
// with c = F Z^T s from the previous pass; q = t + beta q then carries the
// full preconditioned direction, and omega = (Ap, M^-1 Ap) follows its own
// recurrence (den of the previous pass) instead of being summed from q.
// Each pass also sums its s' against the 8 patterns per block (per block of
// threads, folded in a fixed order afterwards); the coarse kernels then form
// c' = F Z^T s', mu = (s', t_D') + (Z^T s', c') and alpha.
//
// Z^T A Z is assembled per solve from 64 FP32 operator products (8 block
// colours x 8 patterns), reduced per block pair in 64-bit fixed point so the
// sums do not depend on the order of the atomics; F comes from a Cholesky
// factorisation (cuSOLVER, loaded at run time) in FP64.
#pragma once

struct CoarseArgs {
  int bs;                // cells per block edge (a multiple of 32)
  int nbx, nby, nbz;     // blocks per axis
  const float* ct;       // c = F Z^T s of the previous pass (K = 8 nbx nby nbz)
  float* hpart;          // per block of threads: [3 z-blocks][2 x-halves][8 patterns]
};
constexpr int CO_ZSLOTS = 3;
constexpr int CO_PART = CO_ZSLOTS * 2 * 8;

// The coarse term of a block as four factors for a row of sign sy:
// (Z c)(x, y, z) = (f0 + sz f1) + sx (f2 + sz f3), patterns p = px + 2 py + 4 pz.
__device__ __forceinline__ void coarse_factors(const CoarseArgs& co, int xb, int yb, int zb, float sy,
                                               float& f0, float& f1, float& f2, float& f3) {
  const float* C = co.ct + ((((long long)zb * co.nby + yb) * co.nbx + xb) << 3);
  f0 = __fmaf_rn(sy, __ldg(C + 2), __ldg(C + 0));
  f1 = __fmaf_rn(sy, __ldg(C + 6), __ldg(C + 4));
  f2 = __fmaf_rn(sy, __ldg(C + 3), __ldg(C + 1));
  f3 = __fmaf_rn(sy, __ldg(C + 7), __ldg(C + 5));
}

// ---------------------------------------------------------------- kernels
// Coarse block (X, Y, Z) and pattern p live at index ((Z nby + Y) nbx + X) 8 + p.

// sign of pattern p at cell (x, y, z)
__device__ __forceinline__ float co_sign(int p, int x, int y, int z) {
  const int par = ((p & 1) ? x : 0) + ((p & 2) ? y : 0) + ((p & 4) ? z : 0);
  return (par & 1) ? -1.0f : 1.0f;
}

// h = Z^T s' of the last pass: the pattern sums its blocks of threads left
// per (z-block, 32-cell half), folded per coarse entry in a fixed order.
// gx, gy, gz, cz: the pass's grid of 64 x 8 x cz-cell blocks.
__global__ void __launch_bounds__(256) k_coarse_fold(CoarseArgs co, int cX, int gx, int gy, int gz, int cz,
                                                     float* h, const PcrState* st) {
  if (st->done) return;
  const int K = co.nbx * co.nby * co.nbz * 8;
  const int m = co.bs >> 5, ry = co.bs >> 3, nHalves = (cX + 31) >> 5;
  for (int j = blockIdx.x * 256 + threadIdx.x; j < K; j += gridDim.x * 256) {
    const int p = j & 7, blk = j >> 3;
    const int X = blk % co.nbx, Y = (blk / co.nbx) % co.nby, Z = blk / (co.nbx * co.nby);
    const int bz0 = (Z * co.bs) / cz, bz1 = min(((Z + 1) * co.bs - 1) / cz, gz - 1);
    double a = 0.0;
    for (int bz = bz0; bz <= bz1; bz++) {
      const int slot = Z - (bz * cz) / co.bs;
      for (int by = Y * ry; by < (Y + 1) * ry && by < gy; by++)
        for (int hx = X * m; hx < (X + 1) * m && hx < nHalves; hx++) {
          const long long bid = (hx >> 1) + (long long)gx * (by + (long long)gy * bz);
          a += co.hpart[bid * CO_PART + slot * 16 + (hx & 1) * 8 + p];
        }
    }
    h[j] = (float)a;
  }
}

// c = F h, one warp per row; with a state: the last block folds h.c and
// forms alpha = delta / ((s', M^-1 s') + 2 beta nu + beta^2 omega), the
// denominator becoming the next omega (set-up pass: (s', M^-1 s') alone).
__global__ void __launch_bounds__(256) k_coarse_matvec(const float* __restrict__ F, const float* __restrict__ h,
                                                       float* c, int K, double* partial, PcrState* st) {
  __shared__ double sred[32];
  if (st && st->done) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double acc = 0.0;
  for (int j = blockIdx.x * 8 + warp; j < K; j += gridDim.x * 8) {
    const float* row = F + (long long)j * K;
    float a = 0.0f;
    for (int i = lane * 4; i < K; i += 128) {
      const float4 f = *reinterpret_cast<const float4*>(row + i);
      const float4 v = *reinterpret_cast<const float4*>(h + i);
      a = __fmaf_rn(f.x, v.x, a);
      a = __fmaf_rn(f.y, v.y, a);
      a = __fmaf_rn(f.z, v.z, a);
      a = __fmaf_rn(f.w, v.w, a);
    }
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) {
      c[j] = a;
      acc += (double)a * (double)h[j];
    }
  }
  if (!st) return;
  const double bsum = block_sum<256>(acc, sred);
  double total;
  if (last_block_sum<256>(bsum, partial, &st->coTicket, gridDim.x * gridDim.y * gridDim.z, &total, sred) &&
      threadIdx.x == 0) {
    const double mu = st->muD + total;
    double den = st->wasSetup ? mu : mu + 2.0 * st->beta * st->nu + st->beta * st->beta * st->omega;
    if (!(den > 0.0)) den = mu;  // rounding guard; (Ap, M^-1 Ap) is positive
    st->alpha = (den > 0.0) ? st->delta / den : 0.0;
    st->omega = den;
    if (!(total == total)) {
      st->status = ESF_ERR_NUMERIC;
      st->done = 1;
    }
  }
}

// h = Z^T v for an FP64 cell vector: one block of threads per coarse block,
// eight sums in a fixed order.
__global__ void __launch_bounds__(256) k_coarse_reduce(GridDev g, CoarseArgs co, const double* __restrict__ v,
                                                       float* h) {
  __shared__ double sred[32];
  const int X = blockIdx.x, Y = blockIdx.y, Z = blockIdx.z;
  const int xa = X * co.bs, ya = Y * co.bs, za = Z * co.bs;
  const int wx = min(co.bs, g.cX - xa), wy = min(co.bs, g.cY - ya), wz = min(co.bs, g.cZ - za);
  const long long n = (long long)wx * wy * wz;
  double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (long long i = threadIdx.x; i < n; i += 256) {
    const int x = xa + (int)(i % wx), y = ya + (int)((i / wx) % wy), z = za + (int)(i / ((long long)wx * wy));
    const double val = v[x + (long long)y * g.cX + (long long)z * g.cslab];
#pragma unroll
    for (int p = 0; p < 8; p++) a[p] += (double)co_sign(p, x, y, z) * val;
  }
  const long long base = (((long long)Z * co.nby + Y) * co.nbx + X) << 3;
#pragma unroll
  for (int p = 0; p < 8; p++) {
    const double t = block_sum<256>(a[p], sred);
    if (threadIdx.x == 0) h[base + p] = (float)t;
  }
}

// r += Z c (the coarse part of the first preconditioned residual)
__global__ void __launch_bounds__(256) k_coarse_add(GridDev g, CoarseArgs co, float* r) {
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < g.R; i += (long long)gridDim.x * 256) {
    const int x = (int)(i % g.cX), y = (int)((i / g.cX) % g.cY), z = (int)(i / g.cslab);
    float f0, f1, f2, f3;
    coarse_factors(co, x / co.bs, y / co.bs, z / co.bs, (y & 1) ? -1.0f : 1.0f, f0, f1, f2, f3);
    const float sz = (z & 1) ? -1.0f : 1.0f, sx = (x & 1) ? -1.0f : 1.0f;
    r[i] += __fmaf_rn(sx, __fmaf_rn(sz, f3, f2), __fmaf_rn(sz, f1, f0));
  }
}

// ---- assembly of E = Z^T A Z
// v = pattern p on the blocks of colour chi (block index parities), 0 elsewhere
__global__ void __launch_bounds__(256) k_coarse_colour(GridDev g, CoarseArgs co, int chi, int p, float* v) {
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < g.R; i += (long long)gridDim.x * 256) {
    const int x = (int)(i % g.cX), y = (int)((i / g.cX) % g.cY), z = (int)(i / g.cslab);
    const int col = ((x / co.bs) & 1) | (((y / co.bs) & 1) << 1) | (((z / co.bs) & 1) << 2);
    v[i] = col == chi ? co_sign(p, x, y, z) : 0.0f;
  }
}

// E[(B', p'), (B, p)] += sum over the cells of B' of sign_p'(cell) y(cell),
// y = A v for v of colour chi and pattern p: a cell of B' takes y from the
// one block B of colour chi whose cells are within one cell of it (B' itself
// when its colour is chi; else the neighbour across the face, edge or
// corner it lies on). Sums over a warp's cells of one (B', B) pair, then
// 64-bit fixed-point atomics (exact, so the order of the atomics does not
// matter).
__global__ void __launch_bounds__(256) k_coarse_gather(GridDev g, CoarseArgs co, int chi, int p,
                                                       const float* __restrict__ y,
                                                       unsigned long long* E, double scale) {
  const int K = co.nbx * co.nby * co.nbz * 8;
  const int nb[3] = {co.nbx, co.nby, co.nbz}, ext[3] = {g.cX, g.cY, g.cZ};
  const long long nWarps = (g.R + 31) / 32;
  const int lane = threadIdx.x & 31;
  for (long long wv = (blockIdx.x * 256LL + threadIdx.x) / 32; wv < nWarps;
       wv += (long long)gridDim.x * 8) {
    const long long i = wv * 32 + lane;
    int key = -1, src = 0, dst = 0;
    float val = 0.0f;
    int c[3] = {0, 0, 0};
    if (i < g.R) {
      c[0] = (int)(i % g.cX);
      c[1] = (int)((i / g.cX) % g.cY);
      c[2] = (int)(i / g.cslab);
      int b[3], d[3];
      bool ok = true;
      for (int a = 0; a < 3; a++) {
        b[a] = c[a] / co.bs;
        const int l = c[a] - b[a] * co.bs, size = min(co.bs, ext[a] - b[a] * co.bs);
        if ((b[a] & 1) == ((chi >> a) & 1)) d[a] = 0;
        else if (l == 0 && b[a] > 0) d[a] = -1;
        else if (l == size - 1 && b[a] + 1 < nb[a]) d[a] = 1;
        else ok = false;
      }
      if (ok) {
        dst = (b[2] * co.nby + b[1]) * co.nbx + b[0];
        src = ((b[2] + d[2]) * co.nby + (b[1] + d[1])) * co.nbx + (b[0] + d[0]);
        key = dst * 27 + (d[0] + 1) + 3 * (d[1] + 1) + 9 * (d[2] + 1);
        val = y[i];
      }
    }
    unsigned live = __ballot_sync(0xffffffffu, key >= 0);
    while (live) {
      const int leader = __ffs(live) - 1;
      const int k = __shfl_sync(0xffffffffu, key, leader);
      const bool mine = key == k;
      const int gd = __shfl_sync(0xffffffffu, dst, leader), gs = __shfl_sync(0xffffffffu, src, leader);
#pragma unroll
      for (int q = 0; q < 8; q++) {
        float t = mine ? co_sign(q, c[0], c[1], c[2]) * val : 0.0f;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == leader) {
          const long long fx = llrint((double)t * scale);
          atomicAdd(E + (long long)(gd * 8 + q) * K + (gs * 8 + p), (unsigned long long)fx);
        }
      }
      live &= ~__ballot_sync(0xffffffffu, mine);
    }
  }
}

// E64 = (E + E^T)/2 from the fixed-point sums; the largest diagonal entry
// (positive) into *dmax as ordered bits
__global__ void __launch_bounds__(256) k_coarse_finish_E(const unsigned long long* E, int K, double inv,
                                                         double* E64, unsigned long long* dmax) {
  for (long long t = blockIdx.x * 256LL + threadIdx.x; t < (long long)K * K; t += (long long)gridDim.x * 256) {
    const int i = (int)(t / K), j = (int)(t % K);
    const double a = (double)(long long)E[t] * inv, b = (double)(long long)E[(long long)j * K + i] * inv;
    const double v = 0.5 * (a + b);
    E64[t] = v;
    if (i == j && v > 0.0) atomicMax(dmax, (unsigned long long)__double_as_longlong(v));
  }
}

__global__ void k_coarse_regularise(double* E64, int K, const unsigned long long* dmax, double eps) {
  const double m = __longlong_as_double((long long)*dmax);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x)
    E64[(long long)i * K + i] += eps * m;
}

// F (row-major, FP32, full) from the inverse's lower triangle (column-major)
__global__ void __launch_bounds__(256) k_coarse_F(const double* inv, int K, float* F) {
  for (long long t = blockIdx.x * 256LL + threadIdx.x; t < (long long)K * K; t += (long long)gridDim.x * 256) {
    const int i = (int)(t / K), j = (int)(t % K);
    F[t] = (float)(i >= j ? inv[i + (long long)j * K] : inv[j + (long long)i * K]);
  }
}

// the largest node m^-1 (positive floats order as their bits)
__global__ void __launch_bounds__(256) k_max_float(const float* v, long long n, unsigned* out) {
  unsigned m = 0;
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < n; i += (long long)gridDim.x * 256) {
    const float x = fabsf(v[i]);
    m = max(m, __float_as_uint(x));
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}
