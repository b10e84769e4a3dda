// Linear algebra of the coupled step on sm_103a:
//  * the matrix-free pressure operator J diag(m^-1) J^T of
//    COUPLED_INTEGRATOR_3D::getMatVecMult (COUPLED_INTEGRATOR_3D.cpp:638-660)
//    as one fused z-marching stencil kernel (no J, no J^T, no mid vector);
//  * the Jacobi-preconditioned Conjugate Residual recurrence of
//    CONJUGATE_RESIDUAL::solvePCR (CONJUGATE_RESIDUAL.inl:109-276) as two
//    kernels per iteration (axpy+norm, update+SpMV+dot) plus a residual check
//    every 5th iteration, with all scalars kept on the device and the
//    iteration chunks replayed as CUDA graphs;
//  * FP32 inner solves inside FP64 iterative refinement (ESF_MIXED), one
//    TMA-staged kernel per inner iteration (esf_pcr_fused.cuh);
//  * the solid system (M + dt^2 K) in 27-neighbour 3x3 block rows.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <chrono>
#include <mutex>
#include <algorithm>
#include <array>
#include <condition_variable>
#include <deque>
#include <map>
#include <thread>
#include <cmath>
#include <type_traits>

#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "esf_common.cuh"

namespace esf {

// ------------------------------------------------------------ reductions
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  __syncthreads();
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x < 32) {
    r = (threadIdx.x < NT / 32) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

// Deposit this block's partial; returns true in the block that arrives last,
// after which `*total` holds the sum of all partials in block order.
template <int NT>
__device__ bool last_block_sum(double mine, double* partial, unsigned int* ticket, int nblocks,
                               double* total, double* sh) {
  __shared__ bool amLast;
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (threadIdx.x == 0) {
    partial[bid] = mine;
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    amLast = (t == (unsigned)nblocks - 1);
  }
  __syncthreads();
  if (!amLast) return false;
  __threadfence();
  double acc = 0;
  for (int i = threadIdx.x; i < nblocks; i += NT) acc += __ldcg(partial + i);
  double s = block_sum<NT>(acc, sh);
  if (threadIdx.x == 0) {
    *total = s;
    *ticket = 0;
  }
  return true;
}

// Scalars after the phase-B reduction r.s (CONJUGATE_RESIDUAL.inl:150-154).
// Reference solves count iterations and leave the stop to the residual check
// every 5th iteration; inner solves of a refinement stop as soon as the
// preconditioned residual's energy r.Ar has fallen by eps^2.
__device__ __forceinline__ void finish_update(PcrState* st, double total) {
  if (st->rebase) {
    // residual replaced by an FP64 recompute: the direction is kept
    st->beta = total / st->delta;
    st->delta = total;
    st->delta0 = total;
    st->rebase = 0;
    st->iter0 = st->iter;
  } else if (st->setup) {
    st->delta = total;
    st->delta0 = total;
    st->beta = 0.0;
    st->setup = 0;
    st->iter0 = st->iter;
    if (st->inner && !(total > 0.0)) {  // zero right-hand side: nothing to do
      st->converged = 1;
      st->done = 1;
    }
  } else {
    st->beta = total / st->delta;
    st->delta = total;
    if (st->inner) {
      st->iter++;
      if (total <= st->eps * st->eps * st->delta0 ||
          (st->cap > 0 && st->iter - st->iter0 >= st->cap)) {
        st->converged = 1;
        st->done = 1;
      }
    } else if (!(st->iter > 0 && st->iter % 5 == 0)) {
      st->iter++;
    }
  }
  if (!(total == total)) {
    st->status = ESF_ERR_NUMERIC;
    st->done = 1;
  }
}

// r - alpha * (Ap / diag), evaluated identically wherever it is formed.
__device__ __forceinline__ double upd_r(double r, double alpha, double ap, double iv) {
  return __fma_rn(-alpha, __dmul_rn(ap, iv), r);
}
__device__ __forceinline__ float upd_r(float r, float alpha, float ap, float iv) {
  return __fmaf_rn(-alpha, __fmul_rn(ap, iv), r);
}

// ------------------------------------------------------- pressure stencil
// Tile of TX x TY cells marching over a z-chunk of CZ cell layers. Per layer:
// (a) each halo cell column forms P = v(k-1)+v(k), Q = v(k-1)-v(k) of the
//     stencil input v; (b) each node forms mid = J^T v from 4 P/Q values,
//     scales by m^-1 and pairs with the previous node layer; (c) each cell
//     forms out = J m from 4 node pairs.  ~36 flops/row, 1 read of v and
//     m^-1, 1 write of out.
constexpr int TX = 32, TY = 8, NT = TX * TY, HX = TX + 2, HY = TY + 2, NXN = TX + 1,
              NYN = TY + 1;
constexpr int NHALO = HX * HY, NNODE = NXN * NYN;

enum StencilMode { S_APPLY = 0, S_UPDATE = 1, S_CHECK = 2, S_RESID_INIT = 3, S_RESID64 = 4 };

template <typename T>
struct StencilArgs {
  const T* in;      // stencil input (APPLY/CHECK/RESID*: x)
  T* x;             // UPDATE: x += alpha d
  const T* d;
  T* r;             // UPDATE: r (read; r - alpha Ap invd is the stencil input); RESID_INIT: out
  const T* Ap;
  const T* invd;
  const T* minv;    // per node, zero on boundary nodes
  T* out;           // APPLY: out; UPDATE: s
  const T* b;       // CHECK / RESID*
  float* out32;     // RESID64: float copy of b - Ax
  double* partial;
  PcrState* st;
};

template <typename T, int MODE>
__global__ void __launch_bounds__(NT) pressure_stencil(GridDev g, StencilArgs<T> a, int cz) {
  __shared__ T sP[NHALO], sQ[NHALO], sV[2][NHALO];
  __shared__ T sA[NNODE], sB[NNODE], sC[NNODE];
  __shared__ double sred[32];
  if (MODE != S_APPLY && a.st->done) return;
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * cz;
  const int z1 = min(z0 + cz, g.cZ);
  T alpha = 0;
  if (MODE == S_UPDATE) alpha = (T)a.st->alpha;

  // halo slots owned by this thread (column offsets into a cell layer)
  long long hc[2];
  bool hin[2], hown[2], hslot[2];
  T prev[2] = {0, 0};
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int hs = tid + q * NT;
    const int hx = hs % HX, hy = hs / HX;
    const int cx = x0 - 1 + hx, cy = y0 - 1 + hy;
    hslot[q] = hs < NHALO;
    hin[q] = hslot[q] && cx >= 0 && cx < g.cX && cy >= 0 && cy < g.cY;
    hown[q] = hin[q] && hx >= 1 && hx <= TX && hy >= 1 && hy <= TY;
    hc[q] = hin[q] ? cx + (long long)cy * g.cX : 0;
  }
  // node slots (boundary nodes carry no unknown: their m^-1 counts as 0)
  long long nc[2];
  bool nok[2], nslot[2];
  T mpx[2] = {0, 0}, mpy[2] = {0, 0}, mpz[2] = {0, 0};
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int ns = tid + q * NT;
    const int nx = x0 + ns % NXN, ny = y0 + ns / NXN;
    nslot[q] = ns < NNODE;
    nok[q] = nslot[q] && nx > 0 && nx < g.X - 1 && ny > 0 && ny < g.Y - 1;
    nc[q] = nok[q] ? nx + (long long)ny * g.X : 0;
  }
  const int ccx = tid % TX, ccy = tid / TX;
  const int cgx = x0 + ccx, cgy = y0 + ccy;
  const bool cin = cgx < g.cX && cgy < g.cY;
  const long long ccol = cgx + (long long)cgy * g.cX;
  double acc = 0.0;
  // r.s of this thread's cells: at most 32 terms, kept in T (the FP64 pipe
  // is a small fraction of the FP32 one) and widened once per thread
  T accT = 0;

  // register prefetch of one layer: stencil input pieces, x and d of the
  // tile's own cells, node m^-1
  T pr[2], pa[2], pi[2], pm[2], px[2], pd[2];
  auto fetch = [&](int kk) {
    const bool layerOk = kk >= 0 && kk < g.cZ;
#pragma unroll
    for (int q = 0; q < 2; q++) {
      pr[q] = 0;
      pa[q] = 0;
      pi[q] = 0;
      px[q] = 0;
      pd[q] = 0;
      if (hin[q] && layerOk) {
        const long long c = hc[q] + (long long)kk * g.cslab;
        if (MODE == S_UPDATE) {
          pr[q] = a.r[c];
          pa[q] = a.Ap[c];
          pi[q] = a.invd[c];
          if (hown[q] && kk >= z0 && kk < z1) {
            px[q] = a.x[c];
            pd[q] = a.d[c];
          }
        } else {
          pr[q] = a.in[c];
        }
      }
      pm[q] = 0;
      if (nok[q] && kk > 0 && kk < g.Z - 1) pm[q] = a.minv[nc[q] + (long long)kk * g.slab];
    }
  };
  fetch(z0 - 1);
  for (int kk = z0 - 1; kk <= z1; kk++) {
    const int vb = kk & 1;
    T cr[2], ca[2], ci[2], cm[2], cxv[2], cdv[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
      cr[q] = pr[q];
      ca[q] = pa[q];
      ci[q] = pi[q];
      cm[q] = pm[q];
      cxv[q] = px[q];
      cdv[q] = pd[q];
    }
    if (kk < z1) fetch(kk + 1);  // in flight while this layer computes
    // (a) stencil input of cell layer kk
#pragma unroll
    for (int q = 0; q < 2; q++) {
      if (!hslot[q]) continue;
      T v = cr[q];
      if (MODE == S_UPDATE) {
        // r itself is advanced by the next phase A: neighbouring tiles read
        // r as halo during this kernel, so it is not written here.
        v = upd_r(cr[q], alpha, ca[q], ci[q]);
        if (hown[q] && kk >= z0 && kk < z1) {
          const long long c = hc[q] + (long long)kk * g.cslab;
          a.x[c] = cxv[q] + alpha * cdv[q];
        }
      }
      const int hs = tid + q * NT;
      sP[hs] = prev[q] + v;
      sQ[hs] = prev[q] - v;
      sV[vb][hs] = prev[q];  // layer kk-1, read in (c) of this layer
      prev[q] = v;
    }
    __syncthreads();
    // (b) node layer kk
    if (kk >= z0) {
#pragma unroll
      for (int q = 0; q < 2; q++) {
        if (!nslot[q]) continue;
        const int ns = tid + q * NT;
        const int nx = ns % NXN, ny = ns / NXN;
        const int s00 = nx + ny * HX, s10 = s00 + 1, s01 = s00 + HX, s11 = s01 + 1;
        T mi = cm[q];
        T mx = ((sP[s00] + sP[s01]) - (sP[s10] + sP[s11])) * mi;
        T my = ((sP[s00] + sP[s10]) - (sP[s01] + sP[s11])) * mi;
        T mz = ((sQ[s00] + sQ[s10]) + (sQ[s01] + sQ[s11])) * mi;
        if (kk >= z0 + 1) {
          sA[ns] = mpx[q] + mx;
          sB[ns] = mpy[q] + my;
          sC[ns] = mz - mpz[q];
        }
        mpx[q] = mx;
        mpy[q] = my;
        mpz[q] = mz;
      }
    }
    __syncthreads();
    // (c) output cell layer kk-1
    if (kk >= z0 + 1 && cin) {
      const int n00 = ccx + ccy * NXN, n10 = n00 + 1, n01 = n00 + NXN, n11 = n01 + 1;
      T xp = (sA[n10] + sA[n11]) - (sA[n00] + sA[n01]);
      T yp = (sB[n01] + sB[n11]) - (sB[n00] + sB[n10]);
      T zp = (sC[n00] + sC[n10]) + (sC[n01] + sC[n11]);
      T o = xp + yp + zp;
      const long long c = ccol + (long long)(kk - 1) * g.cslab;
      if (MODE == S_APPLY) {
        a.out[c] = o;
      } else if (MODE == S_UPDATE) {
        a.out[c] = o;
        T rv = sV[vb][(ccx + 1) + (ccy + 1) * HX];
        accT += rv * o;
      } else if (MODE == S_CHECK) {
        double t = (double)o - (double)a.b[c];
        acc += t * t;
      } else if (MODE == S_RESID_INIT) {
        T bb = a.b[c];
        a.r[c] = (bb - o) * a.invd[c];
        acc += (double)bb * (double)bb;
      } else if (MODE == S_RESID64) {
        T rr = a.b[c] - o;
        a.r[c] = rr;
        a.out32[c] = a.invd ? (float)(rr * a.invd[c]) : (float)rr;
        acc += (double)rr * (double)rr;
      }
    }
  }
  if (MODE == S_APPLY) return;
  if (MODE == S_UPDATE) acc = (double)accT;
  __syncthreads();
  double bs = block_sum<NT>(acc, sred);
  const int nblocks = gridDim.x * gridDim.y * gridDim.z;
  double total;
  if (last_block_sum<NT>(bs, a.partial, &a.st->ticket[1], nblocks, &total, sred) &&
      threadIdx.x == 0) {
    PcrState* st = a.st;
    if (MODE == S_UPDATE) {
      finish_update(st, total);
    } else if (MODE == S_CHECK || MODE == S_RESID64) {
      st->resid2 = total;
      if (MODE == S_CHECK) {
        if (sqrt(total) < st->eps * sqrt(st->bnorm2)) {
          st->converged = 1;
          st->done = 1;
        } else {
          st->iter++;
        }
      }
      if (!(total == total)) {
        st->status = ESF_ERR_NUMERIC;
        st->done = 1;
      }
    } else if (MODE == S_RESID_INIT) {
      st->bnorm2 = total;
    }
  }
}

#include "esf_tma.cuh"
#include "esf_pcr_fused.cuh"

// ------------------------------------------------------- vector kernels
constexpr int VT = 256;

// Phase A of iteration i (CONJUGATE_RESIDUAL.inl:146, 139-142, 156-160):
// [UPDR] r = r - alpha_{i-1} Ap_{i-1}/diag (the residual update of the
// previous iteration); d = beta d + r; Ap = beta Ap + s;
// alpha_i = delta / (Ap . Ap/diag).
template <typename T, bool UPDR>
__global__ void __launch_bounds__(VT) pcr_phase_a(long long n, T* d, T* r, T* Ap, const T* s,
                                                  const T* invd, double* partial, PcrState* st) {
  __shared__ double sred[32];
  if (st->done) return;
  if (st->iter >= st->maxIt) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st->done = 1;
    return;
  }
  const T beta = (T)st->beta;
  const T alpha = (T)st->alpha;
  T acc = 0;
  // four independent element chains per thread keep enough loads in flight
  const long long stride = (long long)gridDim.x * VT;
  long long i = blockIdx.x * (long long)VT + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    T a[4], iv[4], rv[4], dv[4], sv[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const long long j = i + u * stride;
      a[u] = Ap[j];
      iv[u] = invd[j];
      rv[u] = r[j];
      dv[u] = d[j];
      sv[u] = s[j];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const long long j = i + u * stride;
      if (UPDR) {
        rv[u] = upd_r(rv[u], alpha, a[u], iv[u]);
        r[j] = rv[u];
      }
      T dn = beta * dv[u] + rv[u];
      T an = beta * a[u] + sv[u];
      d[j] = dn;
      Ap[j] = an;
      acc += an * (an * iv[u]);
    }
  }
  for (; i < n; i += stride) {
    T a = Ap[i], iv = invd[i], rv = r[i];
    if (UPDR) {
      rv = upd_r(rv, alpha, a, iv);
      r[i] = rv;
    }
    T dv = beta * d[i] + rv;
    T av = beta * a + s[i];
    d[i] = dv;
    Ap[i] = av;
    acc += av * (av * iv);
  }
  double bs = block_sum<VT>((double)acc, sred);
  double total;
  if (last_block_sum<VT>(bs, partial, &st->ticket[0], gridDim.x, &total, sred) &&
      threadIdx.x == 0) {
    st->alpha = (fabs(total) > 0.0) ? st->delta / total : total;
    if (!(total == total)) {
      st->status = ESF_ERR_NUMERIC;
      st->done = 1;
    }
  }
}

// Zero-start set-up for a vector b: r = b/diag, ||b||^2; d = Ap = 0.
template <typename T>
__global__ void __launch_bounds__(VT) pcr_zero_start(long long n, const T* b, const T* invd, T* x,
                                                     T* r, T* d, T* Ap, double* partial,
                                                     PcrState* st) {
  __shared__ double sred[32];
  double acc = 0;
  for (long long i = blockIdx.x * (long long)VT + threadIdx.x; i < n; i += (long long)gridDim.x * VT) {
    T bv = b[i];
    x[i] = 0;
    r[i] = bv * invd[i];
    d[i] = 0;
    Ap[i] = 0;
    acc += (double)bv * (double)bv;
  }
  double bs = block_sum<VT>(acc, sred);
  double total;
  if (last_block_sum<VT>(bs, partial, &st->ticket[2], gridDim.x, &total, sred) &&
      threadIdx.x == 0)
    st->bnorm2 = total;
}

// *out = sum b^2 (deterministic block order)
template <typename T>
__global__ void __launch_bounds__(VT) vec_norm2(long long n, const T* b, double* partial,
                                                unsigned int* ticket, double* out) {
  __shared__ double sred[32];
  double acc = 0;
  for (long long i = blockIdx.x * (long long)VT + threadIdx.x; i < n; i += (long long)gridDim.x * VT)
    acc += (double)b[i] * (double)b[i];
  double bs = block_sum<VT>(acc, sred);
  double total;
  if (last_block_sum<VT>(bs, partial, ticket, gridDim.x, &total, sred) && threadIdx.x == 0)
    *out = total;
}

template <typename T>
__global__ void zero2(long long n, T* a, T* b) {
  for (long long i = blockIdx.x * (long long)VT + threadIdx.x; i < n; i += (long long)gridDim.x * VT) {
    a[i] = 0;
    b[i] = 0;
  }
}

template <typename A, typename B>
__global__ void convert_vec(long long n, const A* in, B* out) {
  for (long long i = blockIdx.x * (long long)VT + threadIdx.x; i < n; i += (long long)gridDim.x * VT)
    out[i] = (B)in[i];
}
// Node m^-1 in FP32 with rows padded to `pitch` floats (a multiple of 4, as
// TMA wants 16-byte row strides); boundary nodes (no unknown) and padding 0.
__global__ void convert_minv_padded(GridDev g, const double* in, float* out, int pitch) {
  const long long n = (long long)pitch * g.Y * g.Z;
  for (long long i = blockIdx.x * (long long)VT + threadIdx.x; i < n; i += (long long)gridDim.x * VT) {
    const int x = (int)(i % pitch);
    const long long yz = i / pitch;
    const int y = (int)(yz % g.Y), z = (int)(yz / g.Y);
    float v = 0.0f;
    if (x > 0 && x < g.X - 1 && y > 0 && y < g.Y - 1 && z > 0 && z < g.Z - 1)
      v = (float)in[x + (long long)y * g.X + (long long)z * g.slab];
    out[i] = v;
  }
}
__global__ void inv_vec(long long n, const double* in, double* out64, float* out32) {
  for (long long i = blockIdx.x * (long long)VT + threadIdx.x; i < n; i += (long long)gridDim.x * VT) {
    double v = 1.0 / in[i];
    if (out64) out64[i] = v;
    if (out32) out32[i] = (float)v;
  }
}
__global__ void add_correction(long long n, double* x, const float* e) {
  for (long long i = blockIdx.x * (long long)VT + threadIdx.x; i < n; i += (long long)gridDim.x * VT)
    x[i] += (double)e[i];
}

static int vec_blocks(long long n) {
  long long b = (n + VT - 1) / VT;
  int cap = 152 * 8;  // 8 resident blocks of 256 threads per SM
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

// ------------------------------------------------------ pressure solver
// Allocations mapped through the driver's virtual-memory calls (vec_alloc),
// released by vec_free.
struct MappedSet {
  struct Mapped {
    CUdeviceptr p;
    size_t size;
    CUmemGenericAllocationHandle h;
  } m[16];
  int n;
};

struct InnerBatcher;
struct PressureWork {
  long long R, T;
  // FP64 path (also the outer loop of the mixed path)
  double *r, *d, *Ap, *s, *invd;
  // mixed inner path
  float *x32, *r32, *d32, *Ap32, *s32, *invd32, *minv32, *b32;
  double* partial;
  PcrState* st;      // device state (FP64 solve / outer loop)
  PcrState* st32;    // device state (inner solve)
  PcrState* hst;     // pinned host copies [8]
  cudaGraphExec_t gFirst, gChunk, gFirst32, gChunk32;
  GridDev g;
  bool graphsFor64, graphsFor32;
  const void* keyA[8];  // pointers the captured graphs were built for
  const void* keyB[8];
  cudaStream_t capStream;
  cudaEvent_t ev[4];
  unsigned long long kFirst, kChunk, kFirst32, kChunk32;  // kernels per graph
  PcrState* stT;  // state used by the kernel timer
  // TMA path of the FP32 update kernel (cells per row a multiple of 4)
  float* minv32p;  // padded node m^-1
  int mpitch;
  TmaMaps tmaps;
  bool tmaOk;
  // one-pass FP32 iteration: second buffer set of r, t = s/diag, q = Ap/diag
  // (the first set is r32, s32, Ap32)
  float *r32b, *s32b, *Ap32b;
  FusedMaps fmaps;
  bool fusedOk;
  // ESF_MIXED_X64: the double-float correction and search direction
  // (allocated on first use) and the graph of its iteration chunk
  float *edf, *ddf;
  cudaGraphExec_t gChunkX;
  unsigned long long kChunkX;
  const void* keyX[8];
  bool graphsForX;
  MappedSet mapped;  // FP32 vectors mapped by vec_alloc
  // inner solves handed to a batcher shared with other scenes or systems
  InnerBatcher* batcher;
  cudaEvent_t batchReady, batchDone;
};

// ---- FP32 vectors of the inner solves in compressible memory. They are
// created with cuMemCreate (compression type GENERIC) and mapped with
// cuMemMap: on GB300 the one-pass iteration runs 8% faster on them (135.5
// against 147.9 us per launch at 256^3, the same with cudaMalloc and with
// non-compressible mapped memory); compression is invisible to the kernels.
// ESF_VMM_COMP=none maps non-compressible memory and =malloc uses
// cudaMalloc (for comparison); any failure of the mapped path falls back to
// cudaMalloc.
struct VmmApi {
  PFN_cuMemGetAllocationGranularity_v10020 gran;
  PFN_cuMemCreate_v10020 create;
  PFN_cuMemAddressReserve_v10020 reserve;
  PFN_cuMemMap_v10020 map;
  PFN_cuMemSetAccess_v10020 access;
  PFN_cuMemUnmap_v10020 unmap;
  PFN_cuMemRelease_v10020 release;
  PFN_cuMemAddressFree_v10020 addrFree;
  bool ok;
};
static const VmmApi& vmm_api() {
  static const VmmApi api = [] {
    VmmApi a;
    memset(&a, 0, sizeof a);
    auto get = [](const char* name, void** fn) {
      cudaDriverEntryPointQueryResult q;
      return cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
             q == cudaDriverEntryPointSuccess && *fn;
    };
    a.ok = get("cuMemGetAllocationGranularity", reinterpret_cast<void**>(&a.gran)) &&
           get("cuMemCreate", reinterpret_cast<void**>(&a.create)) &&
           get("cuMemAddressReserve", reinterpret_cast<void**>(&a.reserve)) &&
           get("cuMemMap", reinterpret_cast<void**>(&a.map)) &&
           get("cuMemSetAccess", reinterpret_cast<void**>(&a.access)) &&
           get("cuMemUnmap", reinterpret_cast<void**>(&a.unmap)) &&
           get("cuMemRelease", reinterpret_cast<void**>(&a.release)) &&
           get("cuMemAddressFree", reinterpret_cast<void**>(&a.addrFree));
    return a;
  }();
  return api;
}
static bool vec_map(MappedSet* w, float** out, size_t bytes, unsigned char comp) {
  const VmmApi& api = vmm_api();
  int dev = 0;
  if (!api.ok || w->n >= 16 || cudaGetDevice(&dev) != cudaSuccess) return false;
  CUmemAllocationProp prop;
  memset(&prop, 0, sizeof prop);
  prop.type = CU_MEM_ALLOCATION_TYPE_PINNED;
  prop.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
  prop.location.id = dev;
  prop.allocFlags.compressionType = comp;
  size_t gran = 0;
  if (api.gran(&gran, &prop, CU_MEM_ALLOC_GRANULARITY_RECOMMENDED) != CUDA_SUCCESS || gran == 0)
    return false;
  MappedSet::Mapped m;
  m.size = (bytes + gran - 1) / gran * gran;
  if (api.create(&m.h, m.size, &prop, 0) != CUDA_SUCCESS) return false;
  if (api.reserve(&m.p, m.size, 0, 0, 0) != CUDA_SUCCESS) {
    api.release(m.h);
    return false;
  }
  CUmemAccessDesc acc;
  memset(&acc, 0, sizeof acc);
  acc.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
  acc.location.id = dev;
  acc.flags = CU_MEM_ACCESS_FLAGS_PROT_READWRITE;
  if (api.map(m.p, m.size, 0, m.h, 0) != CUDA_SUCCESS) {
    api.addrFree(m.p, m.size);
    api.release(m.h);
    return false;
  }
  if (api.access(m.p, m.size, &acc, 1) != CUDA_SUCCESS) {
    api.unmap(m.p, m.size);
    api.addrFree(m.p, m.size);
    api.release(m.h);
    return false;
  }
  w->m[w->n++] = m;
  *out = reinterpret_cast<float*>(m.p);
  return true;
}
static esf_status vec_alloc(MappedSet* w, float** out, size_t bytes) {
  const char* mode = getenv("ESF_VMM_COMP");
  const bool malloc_only = mode && strcmp(mode, "malloc") == 0;
  const unsigned char comp =
      (mode && strcmp(mode, "none") == 0) ? CU_MEM_ALLOCATION_COMP_NONE : CU_MEM_ALLOCATION_COMP_GENERIC;
  if (!malloc_only && vec_map(w, out, bytes, comp)) return ESF_OK;
  ESF_CUDA(cudaMalloc(out, bytes));
  return ESF_OK;
}
static void vec_free(MappedSet* w, float* p) {
  if (!p) return;
  for (int i = 0; i < w->n; i++)
    if (reinterpret_cast<float*>(w->m[i].p) == p) {
      const VmmApi& api = vmm_api();
      api.unmap(w->m[i].p, w->m[i].size);
      api.addrFree(w->m[i].p, w->m[i].size);
      api.release(w->m[i].h);
      w->m[i].p = 0;
      return;
    }
  cudaFree(p);
}

// z-chunk depth: deep enough to amortise the two halo layers, shallow
// enough to give every SM several tiles.
static int stencil_cz(const GridDev& g) {
  long long xy = (long long)((g.cX + TX - 1) / TX) * ((g.cY + TY - 1) / TY);
  long long want = 152LL * 6;
  long long cz = (xy * g.cZ + want - 1) / want;
  if (cz < 4) cz = 4;
  if (cz > 32) cz = 32;
  if (cz > g.cZ) cz = g.cZ;
  return (int)cz;
}
// z-chunk depth of the one-pass iteration: the depth in [4, 64] that best
// trades the last wave's idle block slots (blocks / slots against its
// ceiling) for the two halo layers each chunk re-reads, scored as
// fill x cz / (cz + 4) (at 256^3 this picks 29: 1152 blocks, 1.89 waves of
// 608 slots; a sweep there measured 148 us per launch at 29, 155-157 us at
// 19, 32 and 64, and 165-172 us at 8, 10, 43 and 52). ESF_PRESSURE_CZ
// overrides it, for tuning. The reductions do not follow the register
// kernel's block grid, so any depth gives a valid sum order.
static int fused_cz(const GridDev& g) {
  const char* e = getenv("ESF_PRESSURE_CZ");
  if (e) {
    const int v = atoi(e);
    if (v >= 2) return v < g.cZ ? v : g.cZ;
  }
  static const int slots = [] {
    int dev = 0, sms = 152, per = 4;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pcr_iteration_fused, NT, FU_SMEM) !=
            cudaSuccess ||
        per < 1)
      per = 4;
    return sms * per;
  }();
  const long long cols = (long long)((g.cX + TXW - 1) / TXW) * ((g.cY + TY - 1) / TY);
  // over chunk counts n, each with its balanced depth ceil(cZ / n)
  int best = g.cZ < 4 ? g.cZ : 4;
  double bestScore = -1.0;
  for (int n = 1; n <= g.cZ; n++) {
    const int cz = (g.cZ + n - 1) / n;
    if (cz > 64) continue;
    if (cz < 4) break;
    const long long blocks = cols * ((g.cZ + cz - 1) / cz);
    const double waves = (double)blocks / slots;
    const double fill = waves / std::ceil(waves);
    const double score = fill * cz / (cz + 4.0);
    if (score > bestScore + 1e-12) {
      bestScore = score;
      best = cz;
    }
  }
  return best;
}
template <typename T>
static dim3 stencil_grid(const GridDev& g) {
  int cz = stencil_cz(g);
  return dim3((g.cX + TX - 1) / TX, (g.cY + TY - 1) / TY, (g.cZ + cz - 1) / cz);
}

template <typename T>
esf_status pressure_apply(const GridDev& g, const T* minv, const T* in, T* out, cudaStream_t st) {
  StencilArgs<T> a;
  memset(&a, 0, sizeof a);
  a.in = in;
  a.minv = minv;
  a.out = out;
  ESF_COUNTED pressure_stencil<T, S_APPLY><<<stencil_grid<T>(g), NT, 0, st>>>(g, a, stencil_cz(g));
  ESF_LAUNCH_CHECK();
  return ESF_OK;
}
template esf_status pressure_apply<double>(const GridDev&, const double*, const double*, double*,
                                           cudaStream_t);
template esf_status pressure_apply<float>(const GridDev&, const float*, const float*, float*,
                                          cudaStream_t);

esf_status pressure_work_alloc(PressureWork** out, const GridDev& g, int mixed) {
  PressureWork* w = new PressureWork();
  memset(w, 0, sizeof *w);
  w->R = g.R;
  w->T = g.T;
  w->g = g;
  size_t R = g.R;
  ESF_CUDA(cudaMalloc(&w->r, R * 8));
  ESF_CUDA(cudaMalloc(&w->d, R * 8));
  ESF_CUDA(cudaMalloc(&w->Ap, R * 8));
  ESF_CUDA(cudaMalloc(&w->s, R * 8));
  ESF_CUDA(cudaMalloc(&w->invd, R * 8));
  if (mixed) {
    w->mpitch = (g.X + 3) / 4 * 4;
    float** vecs[] = {&w->x32, &w->r32, &w->d32, &w->Ap32, &w->s32, &w->invd32,
                      &w->b32, &w->r32b, &w->s32b, &w->Ap32b};
    for (float** v : vecs) {
      esf_status e = vec_alloc(&w->mapped, v, R * 4);
      if (e) return e;
    }
    esf_status e = vec_alloc(&w->mapped, &w->minv32p, (size_t)w->mpitch * g.Y * g.Z * 4);
    if (e) return e;
    ESF_CUDA(cudaMalloc(&w->minv32, g.T * 4));
  }
  ESF_CUDA(cudaMalloc(&w->partial, ESF_MAX_PARTIALS * 8));
  ESF_CUDA(cudaMalloc(&w->st, sizeof(PcrState)));
  ESF_CUDA(cudaMalloc(&w->st32, sizeof(PcrState)));
  ESF_CUDA(cudaMalloc(&w->stT, sizeof(PcrState)));
  ESF_CUDA(cudaMemset(w->st, 0, sizeof(PcrState)));
  ESF_CUDA(cudaMemset(w->st32, 0, sizeof(PcrState)));
  ESF_CUDA(cudaMallocHost(&w->hst, 8 * sizeof(PcrState)));
  ESF_CUDA(cudaStreamCreateWithFlags(&w->capStream, cudaStreamNonBlocking));
  for (int i = 0; i < 4; i++) ESF_CUDA(cudaEventCreateWithFlags(&w->ev[i], cudaEventDisableTiming));
  *out = w;
  return ESF_OK;
}

void pressure_work_free(PressureWork* w) {
  if (!w) return;
  cudaFree(w->r); cudaFree(w->d); cudaFree(w->Ap); cudaFree(w->s); cudaFree(w->invd);
  for (float* v : {w->x32, w->r32, w->d32, w->Ap32, w->s32, w->invd32, w->b32, w->r32b, w->s32b,
                   w->Ap32b, w->minv32p})
    vec_free(&w->mapped, v);
  cudaFree(w->minv32);
  cudaFree(w->edf);
  cudaFree(w->ddf);
  cudaFree(w->partial); cudaFree(w->st); cudaFree(w->st32); cudaFree(w->stT);
  if (w->hst) cudaFreeHost(w->hst);
  if (w->gChunkX) cudaGraphExecDestroy(w->gChunkX);
  if (w->gFirst) cudaGraphExecDestroy(w->gFirst);
  if (w->gChunk) cudaGraphExecDestroy(w->gChunk);
  if (w->gFirst32) cudaGraphExecDestroy(w->gFirst32);
  if (w->gChunk32) cudaGraphExecDestroy(w->gChunk32);
  if (w->capStream) cudaStreamDestroy(w->capStream);
  for (int i = 0; i < 4; i++)
    if (w->ev[i]) cudaEventDestroy(w->ev[i]);
  if (w->batcher) pressure_work_set_batcher(w, nullptr);
  if (w->batchReady) cudaEventDestroy(w->batchReady);
  if (w->batchDone) cudaEventDestroy(w->batchDone);
  delete w;
}

// ---- tensor maps of the TMA update kernel
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// 3-D FP32 array [d][h][w] (w a multiple of 4), box bw x bh x 1, zero fill
static esf_status encode3d(CUtensorMap* m, const void* base, long long w, long long h, long long d,
                           unsigned bw, unsigned bh) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = tensor_map_encoder();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return ESF_ERR_CUDA;
  }
  cuuint64_t dims[3] = {(cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)d};
  cuuint64_t strides[2] = {(cuuint64_t)w * 4, (cuuint64_t)w * h * 4};
  cuuint32_t box[3] = {bw, bh, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return ESF_ERR_CUDA;
  }
  return ESF_OK;
}

// FP32 kernels of the mixed path's inner iterations.
enum Fp32Path {
  P32_REGISTER = 0,  // pcr_phase_a + pressure_stencil<float, S_UPDATE>
  P32_TMA = 1,       // pcr_phase_a + pressure_update_tma (same bits as P32_REGISTER)
  P32_FUSED = 2      // pcr_iteration_fused: the whole iteration in one pass
};

// Chooses the FP32 kernels for the mixed path. The TMA kernels need cell
// rows that are a multiple of 4 floats (16-byte row strides); with them the
// one-pass iteration is the default, and ESF_PRESSURE_KERNEL=tma or
// =register selects the two-kernel split with the TMA-staged or the
// register-prefetch update kernel (those two give the same bits; both kept
// for comparison). Converts m^-1 into the padded layout and builds the maps
// once per work.
static esf_status prepare_tma(PressureWork* w, const GridDev& g, const double* minv64,
                              cudaStream_t st, const TmaMaps** out, int* path = nullptr) {
  *out = nullptr;
  if (path) *path = P32_REGISTER;
  const char* pick = getenv("ESF_PRESSURE_KERNEL");
  if (g.cX % 4 != 0 || (pick && strcmp(pick, "register") == 0)) return ESF_OK;
  ESF_COUNTED convert_minv_padded<<<vec_blocks((long long)w->mpitch * g.Y * g.Z), VT, 0, st>>>(
      g, minv64, w->minv32p, w->mpitch);
  ESF_LAUNCH_CHECK();
  if (!w->tmaOk) {
    static const cudaError_t attr = cudaFuncSetAttribute(
        pressure_update_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, TW_SMEM);
    if (attr != cudaSuccess) {
      set_error("pressure_update_tma: %d bytes of shared memory refused: %s", TW_SMEM,
                cudaGetErrorString(attr));
      return ESF_ERR_CUDA;
    }
    TmaMaps m;
    esf_status e;
    if ((e = encode3d(&m.r, w->r32, g.cX, g.cY, g.cZ, TMA_HW, TMA_HH))) return e;
    if ((e = encode3d(&m.ap, w->Ap32, g.cX, g.cY, g.cZ, TMA_HW, TMA_HH))) return e;
    if ((e = encode3d(&m.iv, w->invd32, g.cX, g.cY, g.cZ, TMA_HW, TMA_HH))) return e;
    if ((e = encode3d(&m.x, w->x32, g.cX, g.cY, g.cZ, TXW, TY))) return e;
    if ((e = encode3d(&m.d, w->d32, g.cX, g.cY, g.cZ, TXW, TY))) return e;
    if ((e = encode3d(&m.m, w->minv32p, w->mpitch, g.Y, g.Z, TMA_NW, TMA_NH))) return e;
    w->tmaps = m;
    w->tmaOk = true;
  }
  *out = &w->tmaps;
  if (path) *path = P32_TMA;
  const dim3 gr = tma_grid(g, fused_cz(g));
  const bool fits = (long long)gr.x * gr.y * gr.z * FU_SUMS <= ESF_MAX_PARTIALS / 2;
  if (!path || !fits || (pick && strcmp(pick, "tma") == 0)) return ESF_OK;
  if (!w->fusedOk) {
    static const cudaError_t attr = [] {
      cudaError_t a = cudaFuncSetAttribute(pcr_iteration_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           FU_SMEM);
      if (a != cudaSuccess) return a;
      return cudaFuncSetAttribute(pcr_iteration_fused_x64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  FU_SMEM);
    }();
    if (attr != cudaSuccess) {
      set_error("pcr_iteration_fused: %d bytes of shared memory refused: %s", FU_SMEM,
                cudaGetErrorString(attr));
      return ESF_ERR_CUDA;
    }
    FusedMaps m;
    esf_status e;
    float* rs[2] = {w->r32, w->r32b};
    float* ts[2] = {w->s32, w->s32b};
    float* qs[2] = {w->Ap32, w->Ap32b};
    for (int k = 0; k < 2; k++) {
      if ((e = encode3d(&m.r[k], rs[k], g.cX, g.cY, g.cZ, TMA_HW, TMA_HH))) return e;
      if ((e = encode3d(&m.t[k], ts[k], g.cX, g.cY, g.cZ, TMA_HW, TMA_HH))) return e;
      if ((e = encode3d(&m.q[k], qs[k], g.cX, g.cY, g.cZ, TMA_HW, TMA_HH))) return e;
    }
    if ((e = encode3d(&m.iv, w->invd32, g.cX, g.cY, g.cZ, TXW, TY))) return e;
    if ((e = encode3d(&m.x, w->x32, g.cX, g.cY, g.cZ, TXW, TY))) return e;
    if ((e = encode3d(&m.d, w->d32, g.cX, g.cY, g.cZ, TXW, TY))) return e;
    if ((e = encode3d(&m.m, w->minv32p, w->mpitch, g.Y, g.Z, TMA_NW, TMA_NH))) return e;
    w->fmaps = m;
    w->fusedOk = true;
  }
  *path = P32_FUSED;
  return ESF_OK;
}

// The one-pass FP32 iteration on the work's buffers.
struct FusedKernels {
  GridDev g;
  const FusedMaps* tm;
  FusedPtrs p;
  double* partial;
  PcrState* st;
  float* edf = nullptr;  // set: ESF_MIXED_X64, the double-float correction
  float* ddf = nullptr;  // and direction ((hi, lo) per cell)
  void iteration(cudaStream_t cs) const {
    const int cz = fused_cz(g);
    if (edf) {
      ESF_COUNTED pcr_iteration_fused_x64<<<tma_grid(g, cz), NT, FU_SMEM, cs>>>(g, *tm, p, edf, ddf, partial,
                                                                                st, cz);
      return;
    }
    ESF_COUNTED pcr_iteration_fused<<<tma_grid(g, cz), NT, FU_SMEM, cs>>>(g, *tm, p, partial, st, cz);
  }
  // graph capture interface of PressureKernels (inner solves only)
  void setup_warm(cudaStream_t) const {}
  void setup_zero(cudaStream_t) const {}
  void chunk(cudaStream_t cs, int n, bool) const {
    for (int k = 0; k < n; k++) iteration(cs);
  }
};
static FusedKernels fused_kernels(PressureWork* w, const GridDev& g, PcrState* st) {
  FusedKernels k;
  k.g = g;
  k.tm = &w->fmaps;
  k.p.r[0] = w->r32; k.p.r[1] = w->r32b;
  k.p.t[0] = w->s32; k.p.t[1] = w->s32b;
  k.p.q[0] = w->Ap32; k.p.q[1] = w->Ap32b;
  k.p.x = w->x32;
  k.p.d = w->d32;
  k.partial = w->partial;
  k.st = st;
  return k;
}

// Enqueue iterations of the PCR loop for precision T on stream s.
template <typename T>
struct PressureKernels {
  GridDev g;
  const T *minv, *invd, *b;
  T *x, *r, *d, *Ap, *s;
  double* partial;
  PcrState* st;
  const TmaMaps* tma = nullptr;  // FP32 only: TMA-staged update kernel
  void setup_warm(cudaStream_t cs) const {  // r = (b - Ax)/diag, ||b||; then s = Ar, delta
    StencilArgs<T> a;
    memset(&a, 0, sizeof a);
    a.in = x; a.b = b; a.r = r; a.invd = invd; a.minv = minv; a.partial = partial; a.st = st;
    ESF_COUNTED pressure_stencil<T, S_RESID_INIT><<<stencil_grid<T>(g), NT, 0, cs>>>(g, a, stencil_cz(g));
    ESF_COUNTED zero2<T><<<vec_blocks(g.R), VT, 0, cs>>>(g.R, d, Ap);
    update(cs);
  }
  void setup_zero(cudaStream_t cs) const {
    ESF_COUNTED pcr_zero_start<T><<<vec_blocks(g.R), VT, 0, cs>>>(g.R, b, invd, x, r, d, Ap, partial, st);
    update(cs);
  }
  void phase_a(cudaStream_t cs) const {
    ESF_COUNTED pcr_phase_a<T, true><<<vec_blocks(g.R), VT, 0, cs>>>(g.R, d, r, Ap, s, invd, partial, st);
  }
  void update(cudaStream_t cs) const {
    if constexpr (std::is_same<T, float>::value) {
      if (tma) {
        const int cz = stencil_cz(g);
        ESF_COUNTED pressure_update_tma<<<tma_grid(g, cz), NT, TW_SMEM, cs>>>(g, *tma, x, s, partial, st,
                                                                           cz);
        return;
      }
    }
    StencilArgs<T> a;
    memset(&a, 0, sizeof a);
    a.x = x; a.d = d; a.r = r; a.Ap = Ap; a.invd = invd; a.minv = minv; a.out = s;
    a.partial = partial; a.st = st;
    ESF_COUNTED pressure_stencil<T, S_UPDATE><<<stencil_grid<T>(g), NT, 0, cs>>>(g, a, stencil_cz(g));
  }
  void check(cudaStream_t cs) const {
    StencilArgs<T> a;
    memset(&a, 0, sizeof a);
    a.in = x; a.b = b; a.minv = minv; a.partial = partial; a.st = st;
    ESF_COUNTED pressure_stencil<T, S_CHECK><<<stencil_grid<T>(g), NT, 0, cs>>>(g, a, stencil_cz(g));
  }
  // iterations [i0, i0+n) followed by the residual check of iteration
  // i0+n-1 (reference solves only; inner solves stop on delta)
  void chunk(cudaStream_t cs, int n, bool withCheck) const {
    for (int k = 0; k < n; k++) {
      phase_a(cs);
      update(cs);
    }
    if (withCheck) check(cs);
  }
};

template <typename K>
static esf_status capture(cudaStream_t cs, const K& k, bool first, bool warm, cudaGraphExec_t* exec,
                          unsigned long long* kernels) {
  cudaGraph_t graph;
  *kernels = 0;
  set_capturing(true, kernels);
  cudaError_t ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) {
    set_capturing(false, nullptr);
    ESF_CUDA(ce);
  }
  // reference solves warm-start and check every 5th iteration; inner solves
  // of a refinement start from zero and stop on delta
  if (first) {
    if (warm) k.setup_warm(cs);
    else k.setup_zero(cs);
    k.chunk(cs, 6, warm);  // iterations 0..5, first check at i = 5
  } else {
    k.chunk(cs, 5, warm);  // iterations 5j+1 .. 5j+5
  }
  set_capturing(false, nullptr);
  ESF_CUDA(cudaStreamEndCapture(cs, &graph));
  if (*exec) cudaGraphExecDestroy(*exec);
  ESF_CUDA(cudaGraphInstantiate(exec, graph, 0));
  cudaGraphDestroy(graph);
  return ESF_OK;
}

// Runs one PCR solve from graphs; keeps up to 3 chunks in flight and polls
// pinned copies of the device state.
static esf_status run_graph_solve(PcrState* hst, cudaEvent_t* ev, PcrState* dst,
                                  cudaGraphExec_t gFirst, cudaGraphExec_t gChunk,
                                  unsigned long long kFirst, unsigned long long kChunk, int maxIt,
                                  cudaStream_t st, PcrState* out) {
  const int inflight = 3;
  int launched = 0, waited = 0;
  const int maxChunks = maxIt / 5 + 3;
  bool done = false;
  while (!done) {
    if (launched < maxChunks) {
      const bool first = launched == 0 && gFirst;
      ESF_CUDA(cudaGraphLaunch(first ? gFirst : gChunk, st));
      note_graph_replay(first ? kFirst : kChunk);
      ESF_CUDA(cudaMemcpyAsync(&hst[launched % 4], dst, sizeof(PcrState), cudaMemcpyDeviceToHost, st));
      ESF_CUDA(cudaEventRecord(ev[launched % 4], st));
      launched++;
    }
    if (launched - waited >= inflight || launched >= maxChunks) {
      ESF_CUDA(cudaEventSynchronize(ev[waited % 4]));
      PcrState h = hst[waited % 4];
      waited++;
      if (h.done) {
        done = true;
        *out = h;
      } else if (waited >= maxChunks) {
        done = true;
        *out = h;
      }
    }
  }
  // drain chunks still queued (they exit at once on `done`)
  ESF_CUDA(cudaStreamSynchronize(st));
  ESF_CUDA(cudaMemcpy(out, dst, sizeof(PcrState), cudaMemcpyDeviceToHost));
  return ESF_OK;
}

static esf_status init_state(PcrState* d, double eps, int maxIt, cudaStream_t st, int inner = 0) {
  PcrState h;
  memset(&h, 0, sizeof h);
  h.eps = eps;
  h.maxIt = maxIt;
  h.setup = 1;
  h.inner = inner;
  ESF_CUDA(cudaMemcpyAsync(d, &h, sizeof h, cudaMemcpyHostToDevice, st));
  // the pageable source must not change before the copy runs
  ESF_CUDA(cudaStreamSynchronize(st));
  return ESF_OK;
}

static esf_status batched_inner_solve(PressureWork* w, const GridDev& g, cudaStream_t st, PcrState* out);
static bool batching_pays(PressureWork* w);
static esf_status df_buffers(PressureWork* w, const GridDev& g);

// x += e_hi + e_lo (exact in FP64, then rounded into x), e = 0: the
// double-float correction of an ESF_MIXED_X64 run folded into the solution
__global__ void __launch_bounds__(VT) fold_df(long long n, float2* e, double* x) {
  for (long long i = blockIdx.x * (long long)VT + threadIdx.x; i < n; i += (long long)gridDim.x * VT) {
    const float2 v = e[i];
    x[i] += (double)v.x + (double)v.y;
    e[i] = make_float2(0.0f, 0.0f);
  }
}

esf_status pressure_solve(PressureWork* w, const GridDev& g, const double* minv64,
                          const double* diag64, const double* b, double* x, double eps, int maxIt,
                          int precision, double innerEps, int maxRefine, int* iters,
                          double* relres, int* refinements, int* converged, cudaStream_t st,
                          int* fp64Iters) {
  if (fp64Iters) *fp64Iters = 0;
  {
    dim3 gr = stencil_grid<double>(g);
    if ((long long)gr.x * gr.y * gr.z > ESF_MAX_PARTIALS) return ESF_ERR_UNSUPPORTED;
  }
  ESF_COUNTED inv_vec<<<vec_blocks(g.R), VT, 0, st>>>(g.R, diag64, w->invd, w->invd32);
  ESF_LAUNCH_CHECK();
  // FP64 PCR from the warm start x (the reference's solvePCR): two kernels
  // per iteration replayed as graphs, true-residual check every 5th.
  auto fp64_solve = [&](int itCap, PcrState* out) -> esf_status {
    PressureKernels<double> k{g, minv64, w->invd, b, x, w->r, w->d, w->Ap, w->s, w->partial, w->st};
    const void* key[8] = {minv64, diag64, b, x, nullptr, nullptr, nullptr, nullptr};
    bool rebuild = !w->graphsFor64 || memcmp(key, w->keyA, sizeof key) != 0;
    if (rebuild) {
      esf_status e = capture(w->capStream, k, true, true, &w->gFirst, &w->kFirst);
      if (e) return e;
      e = capture(w->capStream, k, false, true, &w->gChunk, &w->kChunk);
      if (e) return e;
      memcpy(w->keyA, key, sizeof key);
      w->graphsFor64 = true;
    }
    esf_status e = init_state(w->st, eps, itCap, st);
    if (e) return e;
    return run_graph_solve(w->hst, w->ev, w->st, w->gFirst, w->gChunk, w->kFirst, w->kChunk, itCap, st, out);
  };
  if (precision == ESF_FP64) {
    PcrState h;
    esf_status e = fp64_solve(maxIt, &h);
    if (e) return e;
    if (iters) *iters = h.iter;
    if (converged) *converged = h.converged;
    if (refinements) *refinements = 0;
    if (relres) *relres = h.bnorm2 > 0 ? sqrt(h.resid2 / h.bnorm2) : sqrt(h.resid2);
    return h.status ? (esf_status)h.status : ESF_OK;
  }
  // ---- mixed: FP32 inner CR solves (stencil, vectors and updates in FP32,
  // dot products and alpha/beta in FP64) inside FP64 iterative refinement:
  // r = b - A x in FP64; solve A e = r in FP32 from e = 0 until the inner
  // residual energy r.Ar has fallen by innerEps^2, or by the smaller ratio
  // that predicts the outer tolerance; x += e in FP64; repeat until
  // ||b - A x|| < eps ||b||. Capping the inner solves does not work here:
  // short restarted solves stall near 2e-8 on a 256^3 scene, because the
  // slow modes of this operator need long Krylov runs. If the refinements run
  // out before the tolerance is met, FP64 PCR finishes from the refined x.
  // Each inner solve restarts its Krylov space: carrying the direction across
  // the FP64 residual replacement stalls near 1e-7 while the iterate and
  // direction are FP32, whose rounding reaches the residual amplified by the
  // operator's conditioning (ESF_MIXED_X64, above, carries it with both in
  // double-float).
  ESF_COUNTED convert_vec<double, float><<<vec_blocks(g.T), VT, 0, st>>>(g.T, minv64, w->minv32);
  const TmaMaps* tma = nullptr;
  int path = P32_REGISTER;
  {
    esf_status e = prepare_tma(w, g, minv64, st, &tma, &path);
    if (e) return e;
  }
  PressureKernels<float> k32{g, w->minv32, w->invd32, w->b32, w->x32, w->r32, w->d32, w->Ap32,
                             w->s32, w->partial, w->st32};
  k32.tma = tma;
  const bool fused = path == P32_FUSED;
  const FusedKernels kf = fused_kernels(w, g, w->st32);
  const void* key[8] = {w->minv32, w->invd32, w->b32, w->x32, tma, &w->fmaps,
                        reinterpret_cast<const void*>(static_cast<uintptr_t>(path + 1)),
                        reinterpret_cast<const void*>(static_cast<uintptr_t>(fused_cz(g)))};
  if (!w->graphsFor32 || memcmp(key, w->keyB, sizeof key) != 0) {
    esf_status e = fused ? capture(w->capStream, kf, false, false, &w->gChunk32, &w->kChunk32)
                         : capture(w->capStream, k32, false, false, &w->gChunk32, &w->kChunk32);
    if (e) return e;
    memcpy(w->keyB, key, sizeof key);
    w->graphsFor32 = true;
  }
  // start of an inner solve: zero directions (and, one-pass, t of the first
  // buffer set, which the set-up pass reads), then the set-up pass s = A r
  auto inner_setup = [&]() -> esf_status {
    ESF_CUDA(cudaMemsetAsync(w->d32, 0, g.R * 4, st));
    ESF_CUDA(cudaMemsetAsync(w->Ap32, 0, g.R * 4, st));
    if (fused) {
      ESF_CUDA(cudaMemsetAsync(w->s32, 0, g.R * 4, st));
      kf.iteration(st);
    } else {
      k32.update(st);  // s = A r, delta (set-up: alpha = 0)
    }
    ESF_LAUNCH_CHECK();
    return ESF_OK;
  };
  // ||b||
  {
    esf_status e = init_state(w->st, eps, maxIt, st);
    if (e) return e;
  }
  ESF_COUNTED vec_norm2<double><<<vec_blocks(g.R), VT, 0, st>>>(g.R, b, w->partial + ESF_MAX_PARTIALS / 2,
                                                    &w->st->ticket[3], &w->st->bnorm2);
  ESF_LAUNCH_CHECK();
  // r64 = b - A x (FP64), r32 = (b - A x)/diag in FP32, ||r64||^2
  auto true_residual = [&](double* resid2, double* bnorm2) -> esf_status {
    StencilArgs<double> a;
    memset(&a, 0, sizeof a);
    a.in = x; a.b = b; a.r = w->r; a.out32 = w->r32; a.invd = w->invd; a.minv = minv64;
    a.partial = w->partial; a.st = w->st;
    ESF_COUNTED pressure_stencil<double, S_RESID64><<<stencil_grid<double>(g), NT, 0, st>>>(g, a, stencil_cz(g));
    ESF_LAUNCH_CHECK();
    PcrState h;
    ESF_CUDA(cudaMemcpyAsync(&h, w->st, sizeof h, cudaMemcpyDeviceToHost, st));
    ESF_CUDA(cudaStreamSynchronize(st));
    *resid2 = h.resid2;
    *bnorm2 = h.bnorm2;
    return ESF_OK;
  };
  double resid2 = 0, bnorm2 = 0;
  {
    esf_status e = true_residual(&resid2, &bnorm2);
    if (e) return e;
  }
  const double bnorm = sqrt(bnorm2);
  double rel = bnorm > 0 ? sqrt(resid2) / bnorm : sqrt(resid2);
  int total = 0, ref = 0, conv = 0;
  esf_status status = ESF_OK;
  // inner stopping ratio on delta/delta0 for the next inner solve
  auto trigger = [&](double r2) {
    double t = innerEps;
    double target = (r2 > 0) ? 0.5 * eps * bnorm / sqrt(r2) : 0.0;  // predicted convergence
    return (target > t) ? target : t;
  };
  if (!(resid2 == resid2)) {
    status = ESF_ERR_NUMERIC;
  } else if (sqrt(resid2) < eps * bnorm) {
    conv = 1;
  } else if (precision == ESF_MIXED_X64 && fused) {
    // One FP32 Krylov run with its correction e and direction d in
    // double-float (pcr_iteration_fused_x64). The run pauses for an FP64
    // check of ||b - A x|| whenever r.Ar has fallen by 0.1^2 since the last
    // check, or by the ratio that predicts the tolerance if that is larger,
    // or after kX64CheckEvery iterations; it then continues from the checked
    // residual (q and d kept, e folded into x) until a check passes. The
    // recursive FP32 residual drifts from b - A x by the rounding of q
    // (2^-24 of each step), so it is replaced at every check; checking every
    // 10x keeps that drift small against the residual it replaces
    // (replacing a residual that drifted far stalls the run: the recomputed
    // beta swamps the new direction with the old). `refinements` counts the
    // checks.
    constexpr int kX64CheckEvery = 1000;
    {
      esf_status e = df_buffers(w, g);
      if (e) return e;
    }
    FusedKernels kx = kf;
    kx.edf = w->edf;
    kx.ddf = w->ddf;
    const void* keyx[8] = {w->minv32, w->invd32, w->edf, w->ddf, tma, &w->fmaps,
                           reinterpret_cast<const void*>(static_cast<uintptr_t>(fused_cz(g))), nullptr};
    if (!w->graphsForX || memcmp(keyx, w->keyX, sizeof keyx) != 0) {
      esf_status e = capture(w->capStream, kx, false, false, &w->gChunkX, &w->kChunkX);
      if (e) return e;
      memcpy(w->keyX, keyx, sizeof keyx);
      w->graphsForX = true;
    }
    auto predicted = [&](double r2) {
      double t = (r2 > 0) ? 0.5 * eps * bnorm / sqrt(r2) : 0.0;
      t = t > 0.1 ? t : 0.1;
      return t < 0.5 ? t : 0.5;
    };
    ESF_CUDA(cudaMemsetAsync(w->edf, 0, g.R * 8, st));
    ESF_CUDA(cudaMemsetAsync(w->ddf, 0, g.R * 8, st));
    ESF_CUDA(cudaMemsetAsync(w->Ap32, 0, g.R * 4, st));
    ESF_CUDA(cudaMemsetAsync(w->s32, 0, g.R * 4, st));
    PcrState h;
    memset(&h, 0, sizeof h);
    h.eps = predicted(resid2);
    h.maxIt = maxIt;
    h.setup = 1;
    h.inner = 1;
    h.cap = kX64CheckEvery;
    ESF_CUDA(cudaMemcpyAsync(w->st32, &h, sizeof h, cudaMemcpyHostToDevice, st));
    ESF_CUDA(cudaStreamSynchronize(st));
    kx.iteration(st);  // set-up pass: s = A r, delta; d = r; e unchanged (alpha 0)
    ESF_LAUNCH_CHECK();
    for (;;) {
      PcrState hi;
      esf_status e = run_graph_solve(w->hst, w->ev, w->st32, nullptr, w->gChunkX, 0, w->kChunkX, maxIt,
                                     st, &hi);
      if (e) return e;
      total = hi.iter;
      if (hi.status) {
        status = (esf_status)hi.status;
        break;
      }
      // x += e; FP64 residual b - A x, written as (b - A x)/diag into the
      // live r buffer (the recursive FP32 r drifts from it by the rounding
      // of q, 2^-24 of each step); a rebase pass then recomputes t and the
      // scalars from it, keeping q and d
      ESF_COUNTED fold_df<<<vec_blocks(g.R), VT, 0, st>>>(g.R, reinterpret_cast<float2*>(w->edf), x);
      ESF_LAUNCH_CHECK();
      StencilArgs<double> a;
      memset(&a, 0, sizeof a);
      a.in = x; a.b = b; a.r = w->r; a.out32 = (hi.pp & 1) ? w->r32b : w->r32; a.invd = w->invd;
      a.minv = minv64; a.partial = w->partial; a.st = w->st;
      ESF_COUNTED pressure_stencil<double, S_RESID64><<<stencil_grid<double>(g), NT, 0, st>>>(g, a, stencil_cz(g));
      ESF_LAUNCH_CHECK();
      PcrState ho;
      ESF_CUDA(cudaMemcpyAsync(&ho, w->st, sizeof ho, cudaMemcpyDeviceToHost, st));
      ESF_CUDA(cudaStreamSynchronize(st));
      resid2 = ho.resid2;
      ref++;
      rel = bnorm > 0 ? sqrt(resid2) / bnorm : sqrt(resid2);
      if (!(resid2 == resid2)) {
        status = ESF_ERR_NUMERIC;
        break;
      }
      if (sqrt(resid2) < eps * bnorm || resid2 == 0.0) {  // (exact: b = 0 meets no relative test)
        conv = 1;
        break;
      }
      if (total >= maxIt) break;
      hi.done = 0;
      hi.converged = 0;
      hi.rebase = 1;
      hi.eps = predicted(resid2);
      memset(hi.ticket, 0, sizeof hi.ticket);
      ESF_CUDA(cudaMemcpyAsync(w->st32, &hi, sizeof hi, cudaMemcpyHostToDevice, st));
      ESF_CUDA(cudaStreamSynchronize(st));
      kx.iteration(st);  // rebase pass
      ESF_LAUNCH_CHECK();
    }
  } else {
    ESF_CUDA(cudaMemsetAsync(w->x32, 0, g.R * 4, st));
    {
      PcrState h;
      memset(&h, 0, sizeof h);
      h.eps = trigger(resid2);
      h.maxIt = maxIt;
      h.setup = 1;
      h.inner = 1;
      ESF_CUDA(cudaMemcpyAsync(w->st32, &h, sizeof h, cudaMemcpyHostToDevice, st));
      ESF_CUDA(cudaStreamSynchronize(st));
    }
    {
      esf_status e = inner_setup();
      if (e) return e;
    }
    const bool trace = getenv("ESF_TRACE") != nullptr;
    auto t0 = std::chrono::steady_clock::now();
    for (ref = 0; ref < maxRefine; ref++) {
      if (trace) {
        double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        fprintf(stderr, "[esf] refine %d at %.2f ms: iters %d rel %.3e\n", ref, ms, total, rel);
      }
      PcrState hi;
      esf_status e = (fused && batching_pays(w))
                         ? batched_inner_solve(w, g, st, &hi)
                         : run_graph_solve(w->hst, w->ev, w->st32, nullptr, w->gChunk32, 0, w->kChunk32,
                                           maxIt, st, &hi);
      if (e) return e;
      total = hi.iter;
      if (hi.status) {
        status = (esf_status)hi.status;
        break;
      }
      // refinement: fold the FP32 partial solution into x, recompute r
      ESF_COUNTED add_correction<<<vec_blocks(g.R), VT, 0, st>>>(g.R, x, w->x32);
      ESF_CUDA(cudaMemsetAsync(w->x32, 0, g.R * 4, st));
      e = true_residual(&resid2, &bnorm2);
      if (e) return e;
      rel = bnorm > 0 ? sqrt(resid2) / bnorm : sqrt(resid2);
      if (!(resid2 == resid2)) {
        status = ESF_ERR_NUMERIC;
        break;
      }
      if (sqrt(resid2) < eps * bnorm) {
        conv = 1;
        ref++;
        break;
      }
      if (total >= maxIt) break;
      // restart the inner recurrence from the new residual (iteration count
      // carries over; the residual is in the first buffer set)
      hi.done = 0;
      hi.pp = 0;
      hi.converged = 0;
      hi.alpha = 0.0;
      hi.beta = 0.0;
      hi.setup = 1;
      hi.eps = trigger(resid2);
      memset(hi.ticket, 0, sizeof hi.ticket);
      ESF_CUDA(cudaMemcpyAsync(w->st32, &hi, sizeof hi, cudaMemcpyHostToDevice, st));
      ESF_CUDA(cudaStreamSynchronize(st));
      e = inner_setup();
      if (e) return e;
    }
  }
  if (!conv && ref >= maxRefine && status == ESF_OK && total < maxIt) {
    // FP64 finish from the refined iterate
    PcrState h;
    esf_status e = fp64_solve(maxIt - total, &h);
    if (e) return e;
    total += h.iter;
    conv = h.converged;
    rel = h.bnorm2 > 0 ? sqrt(h.resid2 / h.bnorm2) : sqrt(h.resid2);
    if (h.status) status = (esf_status)h.status;
    if (fp64Iters) *fp64Iters = h.iter;
  }
  if (iters) *iters = total;
  if (refinements) *refinements = ref;
  if (relres) *relres = rel;
  if (converged) *converged = conv;
  return status;
}

// Kernel timer: the two per-iteration kernels of the scene's precision on
// scratch vectors seeded from b (the solution x and the solve state are not
// touched), averaged over `reps` launches with CUDA events on `st`.
template <typename T>
static esf_status time_kernels_t(PressureWork* w, const GridDev& g, const T* minv, const T* invd,
                                 const T* bsrc, T* x, T* r, T* d, T* Ap, T* s, int reps,
                                 double* upd, double* ax, cudaStream_t st,
                                 const TmaMaps* tma = nullptr) {
  const long long R = g.R;
  ESF_CUDA(cudaMemcpyAsync(r, bsrc, R * sizeof(T), cudaMemcpyDeviceToDevice, st));
  ESF_CUDA(cudaMemcpyAsync(d, bsrc, R * sizeof(T), cudaMemcpyDeviceToDevice, st));
  ESF_CUDA(cudaMemcpyAsync(Ap, bsrc, R * sizeof(T), cudaMemcpyDeviceToDevice, st));
  ESF_CUDA(cudaMemcpyAsync(s, bsrc, R * sizeof(T), cudaMemcpyDeviceToDevice, st));
  ESF_CUDA(cudaMemsetAsync(x, 0, R * sizeof(T), st));
  PcrState h;
  memset(&h, 0, sizeof h);
  h.alpha = 1e-3;
  h.beta = 1e-3;
  h.delta = 1.0;
  h.iter = 1;
  h.maxIt = 1 << 30;
  h.eps = 0;
  h.inner = 1;
  ESF_CUDA(cudaMemcpyAsync(w->stT, &h, sizeof h, cudaMemcpyHostToDevice, st));
  ESF_CUDA(cudaStreamSynchronize(st));
  PressureKernels<T> k{g, minv, invd, bsrc, x, r, d, Ap, s, w->partial, w->stT};
  k.tma = tma;
  cudaEvent_t e0, e1, e2;
  ESF_CUDA(cudaEventCreate(&e0));
  ESF_CUDA(cudaEventCreate(&e1));
  ESF_CUDA(cudaEventCreate(&e2));
  k.update(st);  // warm-up
  k.phase_a(st);
  ESF_CUDA(cudaEventRecord(e0, st));
  for (int i = 0; i < reps; i++) k.update(st);
  ESF_CUDA(cudaEventRecord(e1, st));
  for (int i = 0; i < reps; i++) k.phase_a(st);
  ESF_CUDA(cudaEventRecord(e2, st));
  ESF_CUDA(cudaEventSynchronize(e2));
  float t1 = 0, t2 = 0;
  cudaEventElapsedTime(&t1, e0, e1);
  cudaEventElapsedTime(&t2, e1, e2);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  *upd = t1 / reps;
  *ax = t2 / reps;
  return ESF_OK;
}

// The double-float correction and direction of ESF_MIXED_X64 (8 bytes a
// row each), allocated on first use.
static esf_status df_buffers(PressureWork* w, const GridDev& g) {
  if (!w->edf) ESF_CUDA(cudaMalloc(&w->edf, g.R * 8));
  if (!w->ddf) ESF_CUDA(cudaMalloc(&w->ddf, g.R * 8));
  return ESF_OK;
}

// The one-pass iteration timed on an inner solve of A e = b from e = 0 (the
// set-up pass and one iteration untimed, then `reps` iterations; the
// tolerance is 0, so every launch does a full iteration).

static esf_status time_fused(PressureWork* w, const GridDev& g, int reps, double* ms,
                             cudaStream_t st, bool x64) {
  const long long R = g.R;
  // x64 (ESF_MIXED_X64): the double-float iteration on zeroed e and d
  if (x64) {
    esf_status e = df_buffers(w, g);
    if (e) return e;
    ESF_CUDA(cudaMemsetAsync(w->edf, 0, R * 8, st));
    ESF_CUDA(cudaMemsetAsync(w->ddf, 0, R * 8, st));
  }
  // r = b/diag in the first buffer set, x = d = q = 0
  ESF_COUNTED pcr_zero_start<float><<<vec_blocks(R), VT, 0, st>>>(R, w->b32, w->invd32, w->x32, w->r32,
                                                               w->d32, w->Ap32, w->partial, w->stT);
  ESF_CUDA(cudaMemsetAsync(w->s32, 0, R * 4, st));
  PcrState h;
  memset(&h, 0, sizeof h);
  h.maxIt = 1 << 30;
  h.setup = 1;
  h.inner = 1;
  ESF_CUDA(cudaMemcpyAsync(w->stT, &h, sizeof h, cudaMemcpyHostToDevice, st));
  ESF_CUDA(cudaStreamSynchronize(st));
  FusedKernels k = fused_kernels(w, g, w->stT);
  if (x64) {
    k.edf = w->edf;
    k.ddf = w->ddf;
  }
  k.iteration(st);
  k.iteration(st);
  cudaEvent_t e0, e1;
  ESF_CUDA(cudaEventCreate(&e0));
  ESF_CUDA(cudaEventCreate(&e1));
  ESF_CUDA(cudaEventRecord(e0, st));
  for (int i = 0; i < reps; i++) k.iteration(st);
  ESF_CUDA(cudaEventRecord(e1, st));
  ESF_CUDA(cudaEventSynchronize(e1));
  float t = 0;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ESF_CUDA(cudaMemcpy(&h, w->stT, sizeof h, cudaMemcpyDeviceToHost));
  if (h.done || h.status) {
    set_error("pressure kernel timer: the timed inner solve stopped early (status %d)", h.status);
    return ESF_ERR_NUMERIC;
  }
  *ms = t / reps;
  return ESF_OK;
}

esf_status pressure_time_kernels(PressureWork* w, const GridDev& g, const double* minv64,
                                 const double* diag64, const double* b, const double* x,
                                 int precision, int reps, double* update_ms, double* axpy_ms,
                                 cudaStream_t st) {
  (void)x;
  ESF_COUNTED inv_vec<<<vec_blocks(g.R), VT, 0, st>>>(g.R, diag64, w->invd, w->invd32);
  if (precision == ESF_MIXED || precision == ESF_MIXED_X64) {
    if (!w->x32) return ESF_ERR_STATE;
    ESF_COUNTED convert_vec<double, float><<<vec_blocks(g.T), VT, 0, st>>>(g.T, minv64, w->minv32);
    ESF_COUNTED convert_vec<double, float><<<vec_blocks(g.R), VT, 0, st>>>(g.R, b, w->b32);
    ESF_LAUNCH_CHECK();
    const TmaMaps* tma = nullptr;
    int path = P32_REGISTER;
    esf_status e = prepare_tma(w, g, minv64, st, &tma, &path);
    if (e) return e;
    if (path == P32_FUSED) {
      *axpy_ms = 0.0;
      return time_fused(w, g, reps, update_ms, st, precision == ESF_MIXED_X64);
    }
    return time_kernels_t<float>(w, g, w->minv32, w->invd32, w->b32, w->x32, w->r32, w->d32,
                                 w->Ap32, w->s32, reps, update_ms, axpy_ms, st, tma);
  }
  // FP64: x scratch is w->s's neighbour; use the FP64 work arrays only
  double* xs = nullptr;
  ESF_CUDA(cudaMalloc(&xs, g.R * 8));
  esf_status e = time_kernels_t<double>(w, g, minv64, w->invd, b, xs, w->r, w->d, w->Ap, w->s, reps,
                                        update_ms, axpy_ms, st);
  cudaStreamSynchronize(st);
  cudaFree(xs);
  return e;
}

// -------------------------------------------------------- solid solver
// Block-row SpMV y = A x over the 27-neighbour 3x3 blocks; modes as for the
// pressure stencil.
template <typename T, int MODE>
__global__ void __launch_bounds__(VT) solid_spmv(long long S, const T* __restrict__ blocks,
                                                 const int* __restrict__ nbr, const T* in,
                                                 const T* b, T* r, T* out, float* out32,
                                                 double* partial, PcrState* st) {
  __shared__ double sred[32];
  if (MODE != S_APPLY && st->done) return;
  double acc = 0;
  T accT = 0;
  for (long long a = blockIdx.x * (long long)VT + threadIdx.x; a < S; a += (long long)gridDim.x * VT) {
    T y0 = 0, y1 = 0, y2 = 0;
    // sliced layout (blk_at/nbr_at): entry je of row a at base + je * 32, so
    // a warp reads 128 contiguous bytes per entry from one region
    const int* nb = nbr + nbr_at(a, 0);
    const T* B0 = blocks + blk_at(a, 0);
    // unrolled by rows of the 3x3x3 neighbourhood so that the loads of nine
    // blocks are in flight together; absent neighbours (m < 0) are skipped,
    // keeping the summation order of the assembled matrix
#pragma unroll 9
    for (int j = 0; j < 27; j++) {
      const int m = __ldg(nb + 32 * j);
      if (m >= 0) {
        const T v0 = in[3 * (long long)m], v1 = in[3 * (long long)m + 1], v2 = in[3 * (long long)m + 2];
        const T* Bj = B0 + 32 * 9 * j;
        y0 += Bj[0] * v0 + Bj[32] * v1 + Bj[64] * v2;
        y1 += Bj[96] * v0 + Bj[128] * v1 + Bj[160] * v2;
        y2 += Bj[192] * v0 + Bj[224] * v1 + Bj[256] * v2;
      }
    }
    T y[3] = {y0, y1, y2};
#pragma unroll
    for (int c = 0; c < 3; c++) {
      long long i = 3 * a + c;
      if (MODE == S_APPLY) {
        out[i] = y[c];
      } else if (MODE == S_UPDATE) {
        out[i] = y[c];
        accT += in[i] * y[c];
      } else if (MODE == S_CHECK) {
        double t = (double)y[c] - (double)b[i];
        acc += t * t;
      } else if (MODE == S_RESID64) {
        T rr = b[i] - y[c];
        r[i] = rr;
        out32[i] = (float)rr;
        acc += (double)rr * (double)rr;
      }
    }
  }
  if (MODE == S_APPLY) return;
  if (MODE == S_UPDATE) acc = (double)accT;
  double bs = block_sum<VT>(acc, sred);
  double total;
  if (last_block_sum<VT>(bs, partial, &st->ticket[1], gridDim.x, &total, sred) &&
      threadIdx.x == 0) {
    if (MODE == S_UPDATE) {
      finish_update(st, total);
    } else {
      st->resid2 = total;
      if (MODE == S_CHECK) {
        if (sqrt(total) < st->eps * sqrt(st->bnorm2)) {
          st->converged = 1;
          st->done = 1;
        } else {
          st->iter++;
        }
      }
      if (!(total == total)) {
        st->status = ESF_ERR_NUMERIC;
        st->done = 1;
      }
    }
  }
}

// ---- matrix-free FP32 stiffness for the solid inner solves (mixed
// precision). The assembled A_s = scale K + diag(damped mass) streams 27
// 3x3 blocks a row (~1 KB); applied cell by cell instead, K x needs per valid
// cell only the corotation R, L, the F-weighted corner gradients GF and
// Jinv dh^3 (43 floats, recorded by the stiffness kernels) and the corners'
// solid DOFs: the element's share for corner m is
//   y_m = scale Jinv dh^3  dPK(dF) . GF_m,   dF = sum_i x_i (x) GF_i,
// with dPK COROTATION::firstPKDifferential (COROTATION.cpp:64-84) as a
// linear map of dF (the map whose value on e_j (x) gf is the stiffness
// kernel's dPK row). Two kernels: one per valid cell writes its 24 shares,
// one per solid node sums the shares of the (up to 8) valid cells around it
// in a fixed order, adds the damped mass and forms the r.s partial of the
// PCR update, as solid_spmv<S_UPDATE> does. The FP64 refinement keeps the
// assembled FP64 matrix for its residual.
struct SolidMF {
  GridDev g;
  long long nc;          // valid cells
  const float* cell;     // MF_PLANES planes of nc floats
  const int* corner;     // 8 planes of nc ints: corner solid DOFs
  const long long* sNode;  // grid node of each solid DOF node
  const int* cellOrd;    // cell -> valid ordinal, or -1
  float mu, lambda, scale;
};
constexpr int MF_CELL_PLANES = 43;

__global__ void __launch_bounds__(VT) k_mf_cell(SolidMF m, const float* __restrict__ x,
                                                 float* __restrict__ share, const PcrState* st) {
  if (st->done) return;
  const long long nc = m.nc;
  for (long long t = blockIdx.x * (long long)VT + threadIdx.x; t < nc; t += (long long)gridDim.x * VT) {
    const float* q = m.cell + t;
    float GF[8][3], dF[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int j = m.corner[i * nc + t];
      float xi[3] = {0.0f, 0.0f, 0.0f};
      if (j >= 0) {
        xi[0] = x[3 * (long long)j];
        xi[1] = x[3 * (long long)j + 1];
        xi[2] = x[3 * (long long)j + 2];
      }
#pragma unroll
      for (int b = 0; b < 3; b++) GF[i][b] = q[(18 + 3 * i + b) * nc];
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) dF[a][b] += xi[a] * GF[i][b];
    }
    float R[3][3], L[3][3];
#pragma unroll
    for (int i = 0; i < 9; i++) {
      R[i / 3][i % 3] = q[i * nc];
      L[i / 3][i % 3] = q[(9 + i) * nc];
    }
    // dPK(dF) = R (2 mu sym + lambda tr(sym) I + lambda tr(R^T dF) I + [L f]x),
    // R^T dF = dFh, sym/skew of dFh, f the axial vector of the skew part
    float h[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) h[a][b] = (R[0][a] * dF[0][b] + R[1][a] * dF[1][b]) + R[2][a] * dF[2][b];
    const float trh = h[0][0] + (h[1][1] + h[2][2]);
    float P[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) P[a][b] = m.mu * (h[a][b] + h[b][a]) + (a == b ? 2.0f * m.lambda * trh : 0.0f);
    const float f[3] = {-0.5f * (h[1][2] - h[2][1]) + 0.5f * (h[2][1] - h[1][2]),
                        -0.5f * (h[2][0] - h[0][2]) + 0.5f * (h[0][2] - h[2][0]),
                        -0.5f * (h[0][1] - h[1][0]) + 0.5f * (h[1][0] - h[0][1])};
    float Lf[3];
#pragma unroll
    for (int a = 0; a < 3; a++) Lf[a] = (L[a][0] * f[0] + L[a][1] * f[1]) + L[a][2] * f[2];
    P[0][1] -= Lf[2];
    P[0][2] += Lf[1];
    P[1][0] += Lf[2];
    P[1][2] -= Lf[0];
    P[2][0] -= Lf[1];
    P[2][1] += Lf[0];
    float D[3][3];  // R P
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) D[a][b] = (R[a][0] * P[0][b] + R[a][1] * P[1][b]) + R[a][2] * P[2][b];
    const float w = q[42 * nc] * m.scale;
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
      for (int r = 0; r < 3; r++)
        share[(3 * i + r) * nc + t] = w * ((D[r][0] * GF[i][0] + D[r][1] * GF[i][1]) + D[r][2] * GF[i][2]);
  }
}

__global__ void __launch_bounds__(VT) k_mf_gather(SolidMF m, long long S, const float* __restrict__ share,
                                                   const float* __restrict__ damped, const float* in, float* out,
                                                   double* partial, PcrState* st) {
  __shared__ double sred[32];
  if (st->done) return;
  const GridDev& g = m.g;
  float accT = 0;
  for (long long a = blockIdx.x * (long long)VT + threadIdx.x; a < S; a += (long long)gridDim.x * VT) {
    const long long n = m.sNode[a];
    const int nx = (int)(n % g.X), ny = (int)((n / g.X) % g.Y), nz = (int)(n / g.slab);
    float y[3] = {0.0f, 0.0f, 0.0f};
    for (int ia = 7; ia >= 0; ia--) {  // the cells around the node, corner ia of each
      const int cx = nx - (ia & 1), cy = ny - ((ia >> 1) & 1), cz = nz - ((ia >> 2) & 1);
      if (cx < 0 || cy < 0 || cz < 0 || cx > g.X - 2 || cy > g.Y - 2 || cz > g.Z - 2) continue;
      const int ord = m.cellOrd[cx + (long long)cy * g.cX + (long long)cz * g.cslab];
      if (ord < 0) continue;
#pragma unroll
      for (int r = 0; r < 3; r++) y[r] += share[(3 * ia + r) * m.nc + ord];
    }
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const long long i = 3 * a + r;
      y[r] += damped[i] * in[i];
      out[i] = y[r];
      accT += in[i] * y[r];
    }
  }
  const double bs = block_sum<VT>((double)accT, sred);
  double total;
  if (last_block_sum<VT>(bs, partial, &st->ticket[1], gridDim.x, &total, sred) && threadIdx.x == 0)
    finish_update(st, total);
}

// x += alpha d; r -= alpha Ap/diag (pointwise part of phase B).
template <typename T>
__global__ void __launch_bounds__(VT) pcr_update_xr(long long n, T* x, const T* d, T* r, const T* Ap,
                                                    const T* invd, const PcrState* st) {
  if (st->done) return;
  const T alpha = (T)st->alpha;
  for (long long i = blockIdx.x * (long long)VT + threadIdx.x; i < n; i += (long long)gridDim.x * VT) {
    x[i] = x[i] + alpha * d[i];
    r[i] = upd_r(r[i], alpha, Ap[i], invd[i]);
  }
}


struct SolidWork {
  long long S;
  PcrState* hst;      // pinned state copies [4]
  cudaEvent_t ev[4];
  // iteration chunks as CUDA graphs, per precision (0 FP64, 1 FP32 inner),
  // recaptured when the system's size or buffers change
  cudaStream_t capStream;
  cudaGraphExec_t gFirst[2], gChunk[2];
  unsigned long long kFirst[2], kChunk[2];
  const void* key[2][16];
  // matrix-free FP32 operator of the inner solves (solid_work_set_matrix_free)
  bool mfOn;
  SolidMF mf;
  float* mfShare;       // 24 planes of the valid cells
  long long mfShareCap;
  float* damped32;      // damped mass (the assembled diagonal's mass part), FP32
  double *r, *d, *Ap, *s, *invd, *partial;
  float *blocks32, *x32, *r32, *d32, *Ap32, *s32, *invd32, *b32;
  PcrState *st, *st32;
  long long cap;
  MappedSet mapped;  // blocks32 in compressible memory (vec_alloc)
};

esf_status solid_work_alloc(SolidWork** out, long long S, int mixed) {
  SolidWork* w = new SolidWork();
  memset(w, 0, sizeof *w);
  w->S = S;
  w->cap = S > 0 ? S : 1;
  size_t n = 3 * w->cap;
  ESF_CUDA(cudaMalloc(&w->r, n * 8));
  ESF_CUDA(cudaMalloc(&w->d, n * 8));
  ESF_CUDA(cudaMalloc(&w->Ap, n * 8));
  ESF_CUDA(cudaMalloc(&w->s, n * 8));
  ESF_CUDA(cudaMalloc(&w->invd, n * 8));
  ESF_CUDA(cudaMalloc(&w->partial, ESF_MAX_PARTIALS * 8));
  ESF_CUDA(cudaMalloc(&w->st, sizeof(PcrState)));
  ESF_CUDA(cudaMalloc(&w->st32, sizeof(PcrState)));
  ESF_CUDA(cudaMallocHost(&w->hst, 4 * sizeof(PcrState)));
  for (int i = 0; i < 4; i++) ESF_CUDA(cudaEventCreateWithFlags(&w->ev[i], cudaEventDisableTiming));
  ESF_CUDA(cudaStreamCreateWithFlags(&w->capStream, cudaStreamNonBlocking));
  if (mixed) {
    // the FP32 blocks in compressible memory: 166 against 171 ms of solid
    // solves per 256^3 step with cudaMalloc
    esf_status e = vec_alloc(&w->mapped, &w->blocks32, rows32(w->cap) * 243 * 4);
    if (e) return e;
    ESF_CUDA(cudaMalloc(&w->x32, n * 4));
    ESF_CUDA(cudaMalloc(&w->r32, n * 4));
    ESF_CUDA(cudaMalloc(&w->d32, n * 4));
    ESF_CUDA(cudaMalloc(&w->Ap32, n * 4));
    ESF_CUDA(cudaMalloc(&w->s32, n * 4));
    ESF_CUDA(cudaMalloc(&w->invd32, n * 4));
    ESF_CUDA(cudaMalloc(&w->b32, n * 4));
  }
  *out = w;
  return ESF_OK;
}
long long solid_work_capacity(const SolidWork* w) { return w ? w->cap : 0; }
void solid_work_free(SolidWork* w) {
  if (!w) return;
  cudaFree(w->r); cudaFree(w->d); cudaFree(w->Ap); cudaFree(w->s); cudaFree(w->invd);
  cudaFree(w->partial); cudaFree(w->st); cudaFree(w->st32);
  vec_free(&w->mapped, w->blocks32);
  cudaFree(w->x32); cudaFree(w->r32); cudaFree(w->d32); cudaFree(w->Ap32); cudaFree(w->s32);
  cudaFree(w->invd32); cudaFree(w->b32);
  if (w->hst) cudaFreeHost(w->hst);
  for (int i = 0; i < 4; i++)
    if (w->ev[i]) cudaEventDestroy(w->ev[i]);
  for (int p = 0; p < 2; p++) {
    if (w->gFirst[p]) cudaGraphExecDestroy(w->gFirst[p]);
    if (w->gChunk[p]) cudaGraphExecDestroy(w->gChunk[p]);
  }
  if (w->capStream) cudaStreamDestroy(w->capStream);
  cudaFree(w->mfShare);
  cudaFree(w->damped32);
  delete w;
}

esf_status solid_work_set_matrix_free(SolidWork* w, const GridDev& g, long long nc, const float* cell,
                                      const int* corner, const long long* sNode, const int* cellOrd,
                                      double mu, double lambda, double scale) {
  if (!w) return ESF_ERR_STATE;
  if (!cell) {
    w->mfOn = false;
    return ESF_OK;
  }
  if (w->mfShareCap < nc) {
    cudaFree(w->mfShare);
    w->mfShare = nullptr;
    w->mfShareCap = 0;
    ESF_CUDA(cudaMalloc(&w->mfShare, (size_t)24 * (nc + nc / 4 + 16) * 4));
    w->mfShareCap = nc + nc / 4 + 16;
  }
  if (!w->damped32) ESF_CUDA(cudaMalloc(&w->damped32, (size_t)3 * w->cap * 4));
  w->mf.g = g;
  w->mf.nc = nc;
  w->mf.cell = cell;
  w->mf.corner = corner;
  w->mf.sNode = sNode;
  w->mf.cellOrd = cellOrd;
  w->mf.mu = (float)mu;
  w->mf.lambda = (float)lambda;
  w->mf.scale = (float)scale;
  w->mfOn = nc > 0;
  return ESF_OK;
}

// The assembled-matrix PCR (CONJUGATE_RESIDUAL.inl:194-276) of the solid
// system: zero start, three kernels per iteration, a residual check every
// 5th iteration for reference solves (inner solves stop on delta).
template <typename T>
struct SolidKernels {
  long long S;
  const T *blocks, *invd, *b;
  const int* nbr;
  T *x, *r, *d, *Ap, *s;
  double* partial;
  PcrState* st;
  // FP32 inner solves: the matrix-free operator instead of the blocks
  const SolidMF* mf = nullptr;
  float* share = nullptr;
  const float* damped = nullptr;
  // s = A r with the r.s partial of the PCR update
  void apply_update(cudaStream_t cs) const {
    if constexpr (std::is_same<T, float>::value) {
      if (mf) {
        ESF_COUNTED k_mf_cell<<<vec_blocks(mf->nc), VT, 0, cs>>>(*mf, r, share, st);
        ESF_COUNTED k_mf_gather<<<vec_blocks(S), VT, 0, cs>>>(*mf, S, share, damped, r, s, partial, st);
        return;
      }
    }
    ESF_COUNTED solid_spmv<T, S_UPDATE><<<vec_blocks(S), VT, 0, cs>>>(S, blocks, nbr, r, nullptr, nullptr, s,
                                                                      nullptr, partial, st);
  }
  void setup_zero(cudaStream_t cs) const {
    const long long n = 3 * S;
    ESF_COUNTED pcr_zero_start<T><<<vec_blocks(n), VT, 0, cs>>>(n, b, invd, x, r, d, Ap, partial, st);
    apply_update(cs);
  }
  void chunk(cudaStream_t cs, int n_it, bool check) const {
    const long long n = 3 * S;
    const int vb = vec_blocks(n), sb = vec_blocks(S);
    for (int k = 0; k < n_it; k++) {
      ESF_COUNTED pcr_phase_a<T, false><<<vb, VT, 0, cs>>>(n, d, r, Ap, s, invd, partial, st);
      ESF_COUNTED pcr_update_xr<T><<<vb, VT, 0, cs>>>(n, x, d, r, Ap, invd, st);
      apply_update(cs);
    }
    if (check)
      ESF_COUNTED solid_spmv<T, S_CHECK><<<sb, VT, 0, cs>>>(S, blocks, nbr, x, b, nullptr, nullptr, nullptr,
                                                            partial, st);
  }
};

template <typename T>
static esf_status capture_solid(cudaStream_t cs, const SolidKernels<T>& k, bool first, bool check,
                                cudaGraphExec_t* exec, unsigned long long* kernels) {
  cudaGraph_t graph;
  *kernels = 0;
  set_capturing(true, kernels);
  cudaError_t ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) {
    set_capturing(false, nullptr);
    ESF_CUDA(ce);
  }
  if (first) {
    k.setup_zero(cs);
    k.chunk(cs, 6, check);  // iterations 0..5, first check at i = 5
  } else {
    k.chunk(cs, 5, check);  // iterations 5j+1 .. 5j+5
  }
  set_capturing(false, nullptr);
  ESF_CUDA(cudaStreamEndCapture(cs, &graph));
  if (*exec) cudaGraphExecDestroy(*exec);
  ESF_CUDA(cudaGraphInstantiate(exec, graph, 0));
  cudaGraphDestroy(graph);
  return ESF_OK;
}

// One solid PCR solve from graphs, set-up and iterations as the reference's.
template <typename T>
static esf_status solid_pcr_graph(SolidWork* w, int slot, long long S, const T* blocks, const int* nbr,
                                  const T* invd, const T* b, T* x, T* r, T* d, T* Ap, T* s,
                                  PcrState* dst, double eps, int maxIt, cudaStream_t st, PcrState* out,
                                  int inner) {
  SolidKernels<T> k{S, blocks, invd, b, nbr, x, r, d, Ap, s, w->partial, dst};
  const bool mf = std::is_same<T, float>::value && w->mfOn;
  if (mf) {
    k.mf = &w->mf;
    k.share = w->mfShare;
    k.damped = w->damped32;
  }
  // the captured graphs hold every pointer and scalar of their launches
  uint64_t mfBits = 0;
  if (mf) {
    const float sc[3] = {w->mf.scale, w->mf.mu, w->mf.lambda};
    uint32_t u[3];
    memcpy(u, sc, sizeof u);
    mfBits = ((uint64_t)u[0] << 32) ^ ((uint64_t)u[1] * 2654435761u) ^ (uint64_t)u[2] ^ (uint64_t)w->mf.nc << 1;
  }
  const void* key[16] = {(const void*)(intptr_t)S, blocks, nbr, invd, b, x, r, d, dst,
                         (const void*)(intptr_t)inner, mf ? w->mf.cell : nullptr, mf ? w->mf.corner : nullptr,
                         mf ? w->mf.cellOrd : nullptr, mf ? (const void*)w->mfShare : nullptr,
                         mf ? (const void*)w->damped32 : nullptr, (const void*)(uintptr_t)mfBits};
  if (!w->gFirst[slot] || memcmp(key, w->key[slot], sizeof key) != 0) {
    esf_status e = capture_solid(w->capStream, k, true, !inner, &w->gFirst[slot], &w->kFirst[slot]);
    if (e) return e;
    e = capture_solid(w->capStream, k, false, !inner, &w->gChunk[slot], &w->kChunk[slot]);
    if (e) return e;
    memcpy(w->key[slot], key, sizeof key);
  }
  esf_status e = init_state(dst, eps, maxIt, st, inner);
  if (e) return e;
  return run_graph_solve(w->hst, w->ev, dst, w->gFirst[slot], w->gChunk[slot], w->kFirst[slot],
                         w->kChunk[slot], maxIt, st, out);
}

esf_status solid_solve(SolidWork* w, long long S, const double* blocks, const int* nbr,
                       const double* diag, const double* b, double* x, double eps, int maxIt,
                       int precision, double innerEps, int maxRefine, int* iters, double* relres,
                       int* refinements, int* converged, cudaStream_t st, const double* damped) {
  if (S <= 0) {
    if (iters) *iters = 0;
    if (converged) *converged = 0;
    if (relres) *relres = 0;
    if (refinements) *refinements = 0;
    return ESF_OK;
  }
  const long long n = 3 * S;
  if ((n + VT - 1) / VT > ESF_MAX_PARTIALS * 64LL) return ESF_ERR_UNSUPPORTED;
  ESF_COUNTED inv_vec<<<vec_blocks(n), VT, 0, st>>>(n, diag, w->invd, w->invd32);
  ESF_LAUNCH_CHECK();
  if (precision == ESF_FP64) {
    PcrState h;
    esf_status e = solid_pcr_graph<double>(w, 0, S, blocks, nbr, w->invd, b, x, w->r, w->d, w->Ap, w->s,
                                           w->st, eps, maxIt, st, &h, 0);
    if (e) return e;
    if (iters) *iters = h.iter;
    if (converged) *converged = h.converged;
    if (refinements) *refinements = 0;
    if (relres) *relres = h.bnorm2 > 0 ? sqrt(h.resid2 / h.bnorm2) : sqrt(h.resid2);
    return h.status ? (esf_status)h.status : ESF_OK;
  }
  // mixed: FP32 blocks, or the matrix-free FP32 operator with the damped mass
  // in FP32; x starts at 0 as in the assembled reference variant
  if (w->mfOn && !damped) {
    set_error("solid_solve: the matrix-free operator needs the damped mass");
    return ESF_ERR_STATE;
  }
  if (w->mfOn) {
    ESF_COUNTED convert_vec<double, float><<<vec_blocks(n), VT, 0, st>>>(n, damped, w->damped32);
  } else {
    ESF_COUNTED convert_vec<double, float><<<vec_blocks(rows32(S) * 243), VT, 0, st>>>(rows32(S) * 243, blocks,
                                                                                     w->blocks32);
  }
  ESF_CUDA(cudaMemsetAsync(x, 0, n * 8, st));
  double bnorm2 = 0;
  {
    esf_status e0 = init_state(w->st, eps, maxIt, st);
    if (e0) return e0;
    ESF_COUNTED vec_norm2<double><<<vec_blocks(n), VT, 0, st>>>(n, b, w->partial, &w->st->ticket[3],
                                                    &w->st->bnorm2);
    PcrState hb;
    ESF_CUDA(cudaMemcpyAsync(&hb, w->st, sizeof hb, cudaMemcpyDeviceToHost, st));
    ESF_CUDA(cudaStreamSynchronize(st));
    bnorm2 = hb.bnorm2;
  }
  int total = 0, ref = 0, conv = 0;
  double rel = 0;
  esf_status status = ESF_OK;
  for (ref = 0; ref <= maxRefine; ref++) {
    init_state(w->st, eps, maxIt, st);
    ESF_COUNTED solid_spmv<double, S_RESID64><<<vec_blocks(S), VT, 0, st>>>(S, blocks, nbr, x, b, w->r,
                                                                nullptr, w->b32, w->partial,
                                                                w->st);
    ESF_LAUNCH_CHECK();
    PcrState h;
    ESF_CUDA(cudaMemcpyAsync(&h, w->st, sizeof h, cudaMemcpyDeviceToHost, st));
    ESF_CUDA(cudaStreamSynchronize(st));
    rel = bnorm2 > 0 ? sqrt(h.resid2 / bnorm2) : sqrt(h.resid2);
    if (!(h.resid2 == h.resid2)) {
      status = ESF_ERR_NUMERIC;
      break;
    }
    if (sqrt(h.resid2) < eps * sqrt(bnorm2)) {
      conv = 1;
      break;
    }
    if (ref == maxRefine || total >= maxIt) break;
    PcrState hi;
    esf_status e = solid_pcr_graph<float>(w, 1, S, w->blocks32, nbr, w->invd32, w->b32, w->x32, w->r32,
                                          w->d32, w->Ap32, w->s32, w->st32, innerEps, maxIt - total,
                                          st, &hi, 1);
    if (e) return e;
    total += hi.iter;
    if (hi.status) {
      status = (esf_status)hi.status;
      break;
    }
    ESF_COUNTED add_correction<<<vec_blocks(n), VT, 0, st>>>(n, x, w->x32);
  }
  if (iters) *iters = total;
  if (refinements) *refinements = ref;
  if (relres) *relres = rel;
  if (converged) *converged = conv;
  return status;
}

// ------------------------------------------- continuous batching (serving)
// The inner FP32 solves of the mixed pressure solves of several scenes (the
// scenes a server is stepping, or the systems of one batched solve),
// advanced in shared launches: one host thread launches chunks of
// pcr_iteration_fused_batch, each chunk five iterations of every task in the
// batch, then gathers the tasks' states into pinned memory. A scene's thread
// hands its inner solve over (after its set-up pass, behind an event on the
// scene's stream) and blocks; the task joins at the next chunk and leaves
// once its state reads done, when the scene's stream is made to wait for
// everything queued on the batch's stream so far. Tasks that finish inside a
// chunk exit the chunk's later launches at once (their state says done): the
// per-scene convergence mask.
// A launch lasts as long as its slowest task, so only scenes of one grid
// shape share launches: each shape has its own lane (stream, tasks, chunks in
// flight), and lanes of different shapes run side by side on the device.
// Up to three chunks are in flight per lane.
// Tile autotuner (opt-in): the depth cz of a block's z-march is the one knob
// of the one-pass kernel's tile. The single-scene heuristic (fused_cz) fills
// the GPU with one scene's blocks; a lane of many small tasks fills it with
// fewer, deeper blocks. With autotuning on, a lane whose task count has
// changed by more than 2x since it was last tuned times two chunks at each
// candidate depth (4, 8, 16, 32, 64 and the whole column, within the partial-
// sum capacity) with CUDA events, then keeps the fastest. Depth changes wait
// until the lane has no chunk in flight. Another depth changes the order of
// the partial sums, so a tuned lane's answers agree with the untuned ones to
// rounding, not bit for bit.
struct InnerBatcher {
  static constexpr int kSlots = FU_MAX_BATCH, kInflight = 3, kRing = 4, kChunk = 5;
  struct Job {
    FusedTask task;
    cudaEvent_t ready = nullptr, done = nullptr;
    bool finished = false;
    PcrState out;
    int slot = -1;
    unsigned long long seq = 0;  // unique per job: a finished job's memory can be reused
  };
  struct Entry {
    Job* job;
    unsigned long long seq;
    int slot;
  };
  struct Chunk {
    int ring;
    unsigned long long order;  // launch order across lanes
    std::vector<Entry> jobs;   // the chunk's tasks in list order
    long long rows;            // pressure rows of its tasks
    int cand;                  // autotuner candidate it measures, or -1
  };
  struct Lane {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[kRing] = {};
    cudaEvent_t t0[kRing] = {}, t1[kRing] = {};  // device time of each chunk's launches
    // autotuner: the lane's depth (0: each task's own), candidates, and the
    // task count it was tuned for
    int cz = 0, tunedTasks = 0, cand = -1, candChunks = 0;
    std::vector<int> cands;
    std::vector<double> candMs;
    PcrState* dStates = nullptr;  // [kRing][kSlots]
    PcrState* hStates = nullptr;  // pinned copies
    std::vector<Job*> active;
    std::deque<Chunk> inflight;
    long long chunks = 0;
  };
  using Shape = std::array<int, 4>;  // cells per axis and the pass's layers per block
  int device = 0;
  FusedTask* dTasks = nullptr;   // device task slots (64-byte aligned)
  FusedTask* hTasks = nullptr;   // pinned staging of the slots
  // a slot is free for a new task when no task holds it and no chunk in
  // flight lists it (lanes run on different streams: a chunk still queued on
  // one lane reads its slots' descriptors when it runs)
  bool slotUsed[kSlots] = {};
  int slotRefs[kSlots] = {};
  std::map<Shape, Lane> lanes;
  std::map<std::array<int, 3>, int> attached;  // works attached, by grid shape (cells per axis)
  std::mutex m;
  std::condition_variable cv, doneCv;
  std::deque<Job*> pending;
  bool stop = false;
  std::thread thr;
  long long launches = 0, taskLaunches = 0, maxTasks = 0, solves = 0;
  long long timedLaunches = 0, timedRows = 0;
  double timedMs = 0;
  bool autotune = false;
  unsigned long long nextSeq = 1, nextOrder = 0;

  static Shape shape_of(const FusedTask& t) { return {t.g.cX, t.g.cY, t.g.cZ, t.cz}; }

  esf_status init(int dev) {
    device = dev;
    cudaSetDevice(dev);
    ESF_CUDA(cudaMalloc(&dTasks, sizeof(FusedTask) * kSlots));
    ESF_CUDA(cudaMallocHost(&hTasks, sizeof(FusedTask) * kSlots));
    static const cudaError_t attr = cudaFuncSetAttribute(
        pcr_iteration_fused_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, FU_SMEM);
    if (attr != cudaSuccess) {
      set_error("pcr_iteration_fused_batch: %d bytes of shared memory refused: %s", FU_SMEM,
                cudaGetErrorString(attr));
      return ESF_ERR_CUDA;
    }
    thr = std::thread([this] { loop(); });
    return ESF_OK;
  }
  esf_status lane_init(Lane& L) {
    ESF_CUDA(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
    for (int i = 0; i < kRing; i++) ESF_CUDA(cudaEventCreateWithFlags(&L.ev[i], cudaEventDisableTiming));
    for (int i = 0; i < kRing; i++) {
      ESF_CUDA(cudaEventCreate(&L.t0[i]));
      ESF_CUDA(cudaEventCreate(&L.t1[i]));
    }
    ESF_CUDA(cudaMalloc(&L.dStates, sizeof(PcrState) * kSlots * kRing));
    ESF_CUDA(cudaMallocHost(&L.hStates, sizeof(PcrState) * kSlots * kRing));
    return ESF_OK;
  }
  void shutdown() {
    {
      std::lock_guard<std::mutex> g(m);
      stop = true;
    }
    cv.notify_all();
    if (thr.joinable()) thr.join();
    cudaSetDevice(device);
    for (auto& kv : lanes) {
      Lane& L = kv.second;
      if (L.stream) cudaStreamSynchronize(L.stream);
      for (int i = 0; i < kRing; i++)
        if (L.ev[i]) cudaEventDestroy(L.ev[i]);
      for (int i = 0; i < kRing; i++) {
        if (L.t0[i]) cudaEventDestroy(L.t0[i]);
        if (L.t1[i]) cudaEventDestroy(L.t1[i]);
      }
      cudaFree(L.dStates);
      if (L.hStates) cudaFreeHost(L.hStates);
      if (L.stream) cudaStreamDestroy(L.stream);
    }
    cudaFree(dTasks);
    if (hTasks) cudaFreeHost(hTasks);
  }
  // called by a scene's thread; blocks until the task is done
  esf_status solve(Job* j) {
    {
      std::lock_guard<std::mutex> g(m);
      if (stop) {
        set_error("inner-solve batcher: stopped");
        return ESF_ERR_STATE;
      }
      j->seq = nextSeq++;
      pending.push_back(j);
    }
    cv.notify_all();
    std::unique_lock<std::mutex> g(m);
    doneCv.wait(g, [&] { return j->finished; });
    return j->out.status == ESF_ERR_CUDA && !j->out.iter ? ESF_ERR_CUDA : ESF_OK;
  }
  // a lane's oldest chunk in flight: read its states, finish the tasks that are done
  void settle(Lane& L) {
    Chunk c = std::move(L.inflight.front());
    L.inflight.pop_front();
    cudaEventSynchronize(L.ev[c.ring]);
    bool any = false;
    std::lock_guard<std::mutex> g(m);
    {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, L.t0[c.ring], L.t1[c.ring]) == cudaSuccess) {
        timedMs += ms;
        timedLaunches += kChunk;
        timedRows += (long long)kChunk * c.rows;
        if (c.cand >= 0 && c.cand == L.cand && c.rows > 0) {
          L.candMs[c.cand] += ms / (double)c.rows;  // per row: task counts can change meanwhile
          L.candChunks++;
        }
      }
    }
    for (size_t i = 0; i < c.jobs.size(); i++) {
      slotRefs[c.jobs[i].slot]--;
      const PcrState& h = L.hStates[c.ring * kSlots + i];
      if (!h.done) continue;
      // only jobs still active are alive; a finished one is not touched
      auto it = std::find(L.active.begin(), L.active.end(), c.jobs[i].job);
      if (it == L.active.end() || (*it)->seq != c.jobs[i].seq) continue;
      Job* j = *it;
      L.active.erase(it);
      // after every chunk queued so far, some of which may still hold the task
      cudaEventRecord(j->done, L.stream);
      slotUsed[j->slot] = false;
      j->out = h;
      j->finished = true;
      solves++;
      any = true;
    }
    if (any) doneCv.notify_all();
  }
  // a task's pass at depth cz (0: its own heuristic depth)
  static void set_depth(FusedTask& t, int cz) {
    if (cz <= 0) cz = fused_cz(t.g);
    t.cz = cz;
    const dim3 gr = tma_grid(t.g, cz);
    t.gx = (int)gr.x;
    t.gy = (int)gr.y;
    t.gz = (int)gr.z;
  }
  // every active task of the lane at depth cz; only with no chunk in flight
  void apply_depth(Lane& L, int cz) {
    L.cz = cz;
    std::lock_guard<std::mutex> g(m);
    for (Job* j : L.active) {
      set_depth(j->task, cz);
      hTasks[j->slot] = j->task;
      cudaMemcpyAsync(dTasks + j->slot, hTasks + j->slot, sizeof(FusedTask), cudaMemcpyHostToDevice,
                      L.stream);
    }
  }
  // The autotuner's step before a lane's next chunk; false while it waits
  // for the lane's chunks in flight to drain before a depth change.
  bool tune(Lane& L) {
    if (!autotune) return true;
    int n;
    GridDev g;
    {
      std::lock_guard<std::mutex> lk(m);
      n = (int)L.active.size();
      if (!n) return true;
      g = L.active[0]->task.g;
    }
    if (L.cand < 0) {
      if (L.tunedTasks && n <= 2 * L.tunedTasks && 2 * n >= L.tunedTasks) return true;
      // start: candidate depths within the partial-sum capacity
      L.cands.clear();
      const long long cols = (long long)((g.cX + TXW - 1) / TXW) * ((g.cY + TY - 1) / TY);
      for (int cz : {4, 8, 16, 32, 64, g.cZ}) {
        if (cz > g.cZ || (!L.cands.empty() && cz <= L.cands.back())) continue;
        if (cols * ((g.cZ + cz - 1) / cz) * FU_SUMS > ESF_MAX_PARTIALS / 2) continue;
        L.cands.push_back(cz);
      }
      if (L.cands.empty()) {
        L.tunedTasks = n;
        return true;
      }
      L.candMs.assign(L.cands.size(), 0.0);
      L.cand = 0;
      L.candChunks = 0;
      L.tunedTasks = n;
    }
    const bool measured = L.candChunks >= 2;
    const int want = measured ? -1 : L.cands[L.cand];
    if (!measured && L.cz == want) return true;
    if (!L.inflight.empty()) return false;  // drain before changing the depth
    if (!measured) {
      apply_depth(L, want);
      return true;
    }
    // this candidate is measured: the next one, or the fastest when done
    if (L.cand + 1 < (int)L.cands.size()) {
      L.cand++;
      L.candChunks = 0;
      apply_depth(L, L.cands[L.cand]);
      return true;
    }
    int best = 0;
    for (int i = 1; i < (int)L.cands.size(); i++)
      if (L.candMs[i] < L.candMs[best]) best = i;
    L.cand = -1;
    apply_depth(L, L.cands[best]);
    return true;
  }
  // one chunk of a lane's active tasks
  void launch(Lane& L) {
    std::vector<Entry> ids;
    FusedBatch b;
    int blocks = 0;
    long long rows = 0;
    {
      std::lock_guard<std::mutex> g(m);
      b.n = (int)L.active.size();
      for (int k = 0; k < b.n; k++) {
        const FusedTask& t = L.active[k]->task;
        b.slot[k] = L.active[k]->slot;
        b.first[k] = blocks;
        blocks += t.gx * t.gy * t.gz;
        rows += t.g.R;
        ids.push_back(Entry{L.active[k], L.active[k]->seq, L.active[k]->slot});
        slotRefs[L.active[k]->slot]++;
      }
    }
    b.first[b.n] = blocks;
    const int ring = (int)(L.chunks % kRing);
    cudaEventRecord(L.t0[ring], L.stream);
    for (int k = 0; k < kChunk; k++) {
      ESF_COUNTED pcr_iteration_fused_batch<<<blocks, NT, FU_SMEM, L.stream>>>(dTasks, b);
    }
    cudaEventRecord(L.t1[ring], L.stream);
    ESF_COUNTED gather_task_states<<<1, 64, 0, L.stream>>>(dTasks, b, L.dStates + ring * kSlots);
    cudaMemcpyAsync(L.hStates + ring * kSlots, L.dStates + ring * kSlots, sizeof(PcrState) * b.n,
                    cudaMemcpyDeviceToHost, L.stream);
    cudaEventRecord(L.ev[ring], L.stream);
    L.chunks++;
    launches += kChunk;
    taskLaunches += (long long)kChunk * b.n;
    if (b.n > maxTasks) maxTasks = b.n;
    L.inflight.push_back(Chunk{ring, nextOrder++, std::move(ids), rows, L.cand});
  }
  void loop() {
    cudaSetDevice(device);
    for (;;) {
      std::vector<Job*> joining;
      {
        std::unique_lock<std::mutex> g(m);
        bool busy = false;
        for (auto& kv : lanes) busy = busy || !kv.second.active.empty() || !kv.second.inflight.empty();
        if (!busy) cv.wait(g, [&] { return stop || !pending.empty(); });
        if (stop && pending.empty() && !busy) return;
        while (!pending.empty()) {
          int s = 0;
          while (s < kSlots && (slotUsed[s] || slotRefs[s] > 0)) s++;
          if (s == kSlots) break;  // wait for chunks in flight to release slots
          Job* j = pending.front();
          pending.pop_front();
          slotUsed[s] = true;
          j->slot = s;
          joining.push_back(j);
        }
      }
      for (Job* j : joining) {
        Lane& L = lanes[shape_of(j->task)];
        if (!L.stream && lane_init(L) != ESF_OK) {
          std::lock_guard<std::mutex> g(m);
          memset(&j->out, 0, sizeof j->out);
          j->out.status = ESF_ERR_CUDA;
          j->out.done = 1;
          j->finished = true;
          slotUsed[j->slot] = false;
          doneCv.notify_all();
          continue;
        }
        if (L.cz) set_depth(j->task, L.cz);
        hTasks[j->slot] = j->task;
        cudaMemcpyAsync(dTasks + j->slot, hTasks + j->slot, sizeof(FusedTask), cudaMemcpyHostToDevice,
                        L.stream);
        cudaStreamWaitEvent(L.stream, j->ready, 0);
        std::lock_guard<std::mutex> g(m);
        L.active.push_back(j);
      }
      // a chunk on every lane that has tasks and room; settle what is ready
      bool launched = false;
      for (auto& kv : lanes) {
        Lane& L = kv.second;
        while (!L.inflight.empty() && cudaEventQuery(L.ev[L.inflight.front().ring]) == cudaSuccess)
          settle(L);
        bool has;
        {
          std::lock_guard<std::mutex> g(m);
          has = !L.active.empty();
        }
        if (has && (int)L.inflight.size() < kInflight && tune(L)) {
          launch(L);
          launched = true;
        }
      }
      if (!launched) {
        // every lane is full or idle: wait for the oldest chunk in flight
        Lane* oldest = nullptr;
        for (auto& kv : lanes)
          if (!kv.second.inflight.empty() &&
              (!oldest || kv.second.inflight.front().order < oldest->inflight.front().order))
            oldest = &kv.second;
        if (oldest) settle(*oldest);
      }
    }
  }
};

esf_status batcher_create(int device, InnerBatcher** out, bool autotune) {
  InnerBatcher* b = new InnerBatcher();
  b->autotune = autotune;
  esf_status e = b->init(device);
  if (e) {
    b->shutdown();
    delete b;
    return e;
  }
  *out = b;
  return ESF_OK;
}
void batcher_destroy(InnerBatcher* b) {
  if (!b) return;
  b->shutdown();
  delete b;
}
void batcher_stats(InnerBatcher* b, esf_batch_stats* out) {
  std::lock_guard<std::mutex> g(b->m);
  out->launches = b->launches;
  out->task_launches = b->taskLaunches;
  out->max_tasks = b->maxTasks;
  out->inner_solves = b->solves;
  out->timed_launches = b->timedLaunches;
  out->timed_rows = b->timedRows;
  out->timed_ms = b->timedMs;
}
esf_status pressure_work_set_batcher(PressureWork* w, InnerBatcher* b) {
  if (!w) return ESF_ERR_STATE;
  if (b && !w->batchReady) {
    ESF_CUDA(cudaEventCreateWithFlags(&w->batchReady, cudaEventDisableTiming));
    ESF_CUDA(cudaEventCreateWithFlags(&w->batchDone, cudaEventDisableTiming));
  }
  const std::array<int, 3> shape = {w->g.cX, w->g.cY, w->g.cZ};
  if (w->batcher) {
    std::lock_guard<std::mutex> g(w->batcher->m);
    w->batcher->attached[shape]--;
  }
  w->batcher = b;
  if (b) {
    std::lock_guard<std::mutex> g(b->m);
    b->attached[shape]++;
  }
  return ESF_OK;
}
// Whether a scene's inner solves go through its batcher: only for a grid
// whose own pass fills at most a quarter of the GPU's resident blocks (a
// larger one already keeps the GPU busy alone, and the batcher's
// one-launch-at-a-time host loop and its kernel's spills only cost; measured
// on the 48^3-160^3 serving mix: 6.9 scene-steps/s batching every shape
// against 7.6 unbatched), and only while another work of the same grid shape
// is attached (a task alone in its lane gains nothing over the scene's own
// captured graphs).
static bool batching_pays(PressureWork* w) {
  if (!w->batcher) return false;
  static const int slots = [] {
    int dev = 0, sms = 152, per = 4;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pcr_iteration_fused_batch, NT, FU_SMEM) !=
            cudaSuccess ||
        per < 1)
      per = 4;
    return sms * per;
  }();
  const dim3 gr = tma_grid(w->g, fused_cz(w->g));
  if ((long long)gr.x * gr.y * gr.z * 4 > slots) return false;
  std::lock_guard<std::mutex> g(w->batcher->m);
  auto it = w->batcher->attached.find({w->g.cX, w->g.cY, w->g.cZ});
  return it != w->batcher->attached.end() && it->second >= 2;
}

// One inner solve of a scene through the batcher: the set-up pass has been
// queued on the scene's stream; the task joins the batch behind it, and the
// scene's stream resumes behind the batch stream's work once it is done.
static esf_status batched_inner_solve(PressureWork* w, const GridDev& g, cudaStream_t st, PcrState* out) {
  InnerBatcher::Job j;
  const FusedKernels kf = fused_kernels(w, g, w->st32);
  j.task.tm = w->fmaps;
  j.task.g = g;
  j.task.p = kf.p;
  j.task.partial = w->partial;
  j.task.st = w->st32;
  j.task.cz = fused_cz(g);
  const dim3 gr = tma_grid(g, j.task.cz);
  j.task.gx = (int)gr.x;
  j.task.gy = (int)gr.y;
  j.task.gz = (int)gr.z;
  j.ready = w->batchReady;
  j.done = w->batchDone;
  ESF_CUDA(cudaEventRecord(j.ready, st));
  {
    esf_status e = w->batcher->solve(&j);
    if (e) return e;
  }
  ESF_CUDA(cudaStreamWaitEvent(st, j.done, 0));
  *out = j.out;
  return ESF_OK;
}

// ------------------------------------------------- bounded-wait self-test
// One thread arms an mbarrier for a 16-byte copy that is never issued and
// waits on it with mbar_wait, the TMA kernels' bounded wait (TMA_WAIT_LIMIT
// polls). The phase never completes, so the wait runs out; the thread
// records that in *gaveUp, invalidates the barrier and the block returns.
// No copy is in flight, so nothing writes the barrier's shared memory after
// the block has ended.
__global__ void k_selftest_mbar_wait(int* gaveUp) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_expect_tx(&bar, 16);
    const bool landed = mbar_wait(&bar, 0);
    *gaveUp = landed ? 0 : 1;
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bar)) : "memory");
  }
}

esf_status selftest_mbar_wait(int* gaveUp, cudaStream_t st) {
  ESF_COUNTED k_selftest_mbar_wait<<<1, 32, 0, st>>>(gaveUp);
  ESF_LAUNCH_CHECK();
  return ESF_OK;
}

// ------------------------------------ allocation-free FP64 pressure solve
// Scratch of esf_pressure_solve_static: one file-scope device array, carved
// into [PcrState | block partials | invd r d Ap s], sized for grids of at
// most ESF_STATIC_SOLVE_MAX_CELLS cells (10.1 MiB). It is part of the
// module image, so no call allocates device or pinned memory, creates a
// stream, event or graph, or frees anything.
constexpr long long kStaticPartials = 16384;
constexpr size_t kStaticStateBytes = 256;
constexpr size_t kStaticScratchBytes =
    kStaticStateBytes + kStaticPartials * 8 + 5ull * ESF_STATIC_SOLVE_MAX_CELLS * 8;
static_assert(sizeof(PcrState) <= kStaticStateBytes, "PcrState outgrew its slot");
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// The context the calling thread has current, by its process-unique ID
// (cuCtxGetId); false when there is none or it has been destroyed.
static bool current_context_id(unsigned long long* id) {
  struct Api {
    PFN_cuCtxGetCurrent_v4000 current = nullptr;
    PFN_cuCtxGetId_v12000 getId = nullptr;
  };
  static const Api api = [] {
    Api a;
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      a.current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      a.getId = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
    return a;
  }();
  CUcontext ctx = nullptr;
  if (!api.current || !api.getId || api.current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return api.getId(ctx, id) == CUDA_SUCCESS;
}

// Device address of g_static_scratch on the current device. In host code the
// array's name is only a stand-in, so the address comes from
// cudaGetSymbolAddress, called with the device current: once per device, and
// again whenever the device's context has been re-created since (after a
// cudaDeviceReset the module is loaded anew and the array can move), which
// the context's ID tells. The lookup allocates nothing; it can load the
// module's device code.
esf_status static_scratch_address(void** out) {
  static std::mutex mu;
  static unsigned long long ctxOf[ESF_STATIC_SOLVE_MAX_DEVICES];
  static void* addrOf[ESF_STATIC_SOLVE_MAX_DEVICES];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ESF_ERR_CUDA;
  if (dev < 0 || dev >= ESF_STATIC_SOLVE_MAX_DEVICES) {
    set_error("esf_pressure_solve_static: device %d beyond the %d supported", dev,
              ESF_STATIC_SOLVE_MAX_DEVICES);
    return ESF_ERR_UNSUPPORTED;
  }
  unsigned long long id = 0;
  const bool known = current_context_id(&id);
  std::lock_guard<std::mutex> lock(mu);
  if (known && addrOf[dev] && ctxOf[dev] == id) {
    *out = addrOf[dev];
    return ESF_OK;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
  if (e != cudaSuccess || !p) {
    set_error("esf_pressure_solve_static: cudaGetSymbolAddress failed on device %d: %s", dev,
              cudaGetErrorString(e));
    return ESF_ERR_CUDA;
  }
  // cache only under the context the lookup ran in; without an ID, look up
  // again on the next call
  addrOf[dev] = current_context_id(&id) ? p : nullptr;
  ctxOf[dev] = id;
  *out = p;
  return ESF_OK;
}

// The reference's FP64 solvePCR with the kernels of the graph path, launched
// one by one: set-up, iterations 0..5 and their residual check, then chunks
// of 5 iterations + check, the state polled after every 4 chunks (kernels
// queued after convergence exit at once, as in the graph path). Same kernels
// in the same order as esf_pressure_solve at ESF_FP64, so the same bits.
esf_status pressure_solve_static(void* scratch, const GridDev& g, const double* minv,
                                 const double* diag, const double* b, double* x, double eps,
                                 int maxIt, int* iters, double* relres, int* converged,
                                 cudaStream_t st) {
  if (g.R > ESF_STATIC_SOLVE_MAX_CELLS) {
    set_error("esf_pressure_solve_static: grid has %lld cells, the static scratch holds at most %d",
              g.R, ESF_STATIC_SOLVE_MAX_CELLS);
    return ESF_ERR_UNSUPPORTED;
  }
  {
    dim3 gr = stencil_grid<double>(g);
    long long nb = (long long)gr.x * gr.y * gr.z;
    if (nb > kStaticPartials) {
      set_error("esf_pressure_solve_static: grid needs %lld stencil blocks, the static scratch holds "
                "%lld partial sums", nb, kStaticPartials);
      return ESF_ERR_UNSUPPORTED;
    }
  }
  unsigned char* base = static_cast<unsigned char*>(scratch);
  PcrState* state = reinterpret_cast<PcrState*>(base);
  double* partial = reinterpret_cast<double*>(base + kStaticStateBytes);
  double* vec = partial + kStaticPartials;
  const long long R = g.R;
  double *invd = vec, *r = vec + R, *d = vec + 2 * R, *Ap = vec + 3 * R, *s = vec + 4 * R;
  ESF_COUNTED inv_vec<<<vec_blocks(R), VT, 0, st>>>(R, diag, invd, nullptr);
  ESF_LAUNCH_CHECK();
  // zeroes the whole state (tickets included) before any kernel reads it;
  // set-up zeroes d and Ap
  {
    esf_status e = init_state(state, eps, maxIt, st);
    if (e) return e;
  }
  PressureKernels<double> k{g, minv, invd, b, x, r, d, Ap, s, partial, state};
  k.setup_warm(st);
  k.chunk(st, 6, true);
  ESF_LAUNCH_CHECK();
  const int maxChunks = maxIt / 5 + 3;
  int launched = 1;
  PcrState h;
  for (;;) {
    ESF_CUDA(cudaMemcpyAsync(&h, state, sizeof h, cudaMemcpyDeviceToHost, st));
    ESF_CUDA(cudaStreamSynchronize(st));
    if (h.done || launched >= maxChunks) break;
    for (int c = 0; c < 4 && launched < maxChunks; c++, launched++) k.chunk(st, 5, true);
    ESF_LAUNCH_CHECK();
  }
  if (iters) *iters = h.iter;
  if (converged) *converged = h.converged;
  if (relres) *relres = h.bnorm2 > 0 ? sqrt(h.resid2 / h.bnorm2) : sqrt(h.resid2);
  return h.status ? (esf_status)h.status : ESF_OK;
}

}  // namespace esf
