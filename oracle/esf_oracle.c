/*
 * esf_oracle.c - CPU restatement of EULERSF's per-timestep coupled
 * solid-fluid step (yunteng/EULERSF). TEST INFRASTRUCTURE ONLY: the checker
 * for the CUDA implementation, never part of the product (see esf_oracle.h).
 *
 * Every function names the reference file:line it restates. Arithmetic is
 * written in the reference's operation order (Eigen 3.2.6 evaluation order
 * for the 3x3 determinant/inverse, sequential sums, the 4-lane SSE2 order of
 * VectorXd dot products) so that the oracle tracks the reference build to
 * rounding. Build with -ffp-contract=off: the reference is compiled for
 * x86-64 without FMA, and an aarch64 compiler would otherwise fuse a*b+c.
 *
 * Differences from the reference, all deliberate:
 *  - the symmetric 3x3 eigen-decomposition of F^T F (Eigen::JacobiSVD in
 *    COROTATION.cpp:239) is a cyclic Jacobi eigen-solver; R, S and L are
 *    invariant to its sign/order choices, so stress agrees to rounding;
 *  - solid-solid particle contact (DEFOR_SOLID_3D.cpp:969-995) needs the
 *    DT-Grid rest SDF and is not restated: a particle inside another solid's
 *    narrow band raises the report status instead (single-solid scenes never
 *    reach it);
 *  - the BVH broad phase (TRIANGLE_BVH.cpp:90-98) is restated by its result:
 *    the root box is the vertex AABB, and two BVHs collide iff some pair of
 *    triangle boxes overlaps.
 */
#include "esf_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAXS ESF_MAX_SOLIDS

static inline double dmin(double a, double b) { return (b < a) ? b : a; } /* std::min */
static inline double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max */
/* Eigen's unrolled 3-term sum (Redux.h redux_novec_unroller): a + (b + c). */
static inline double sum3(double a, double b, double c) { return a + (b + c); }
static inline int imin(int a, int b) { return (b < a) ? b : a; }
static inline int imax(int a, int b) { return (a < b) ? b : a; }

/* ------------------------------------------------------------ MT19937 ---- */
/* MERSENNETWISTER (include/util/MERSENNETWISTER.h:137-262): standard
 * MT19937; rand() = randInt() * (1/4294967295.0) (:146-150). */
typedef struct {
  uint32_t mt[624];
  int idx;
} mt19937;

static void mt_seed(mt19937* m, uint32_t seed) {
  m->mt[0] = seed;
  for (int i = 1; i < 624; i++)
    m->mt[i] = 1812433253u * (m->mt[i - 1] ^ (m->mt[i - 1] >> 30)) + (uint32_t)i;
  m->idx = 624;
}
static void mt_twist(mt19937* m) {
  for (int i = 0; i < 624; i++) {
    uint32_t y = (m->mt[i] & 0x80000000u) | (m->mt[(i + 1) % 624] & 0x7fffffffu);
    m->mt[i] = m->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
  }
  m->idx = 0;
}
static uint32_t mt_next(mt19937* m) {
  if (m->idx >= 624) mt_twist(m);
  uint32_t y = m->mt[m->idx++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}
static double mt_rand(mt19937* m, double n) {
  return ((double)mt_next(m) * (1.0 / 4294967295.0)) * n;
}
void esfo_mt19937(uint32_t seed, uint32_t* out, long n) {
  mt19937 m;
  mt_seed(&m, seed);
  for (long i = 0; i < n; i++) out[i] = mt_next(&m);
}

/* ---------------------------------------------------------- 3x3 algebra -- */
typedef struct { double m[3][3]; } m3;

static m3 m3_mul(const m3* a, const m3* b) {
  m3 r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      r.m[i][j] = (a->m[i][0] * b->m[0][j] + a->m[i][1] * b->m[1][j]) + a->m[i][2] * b->m[2][j];
  return r;
}
static m3 m3_mul_bt(const m3* a, const m3* b) { /* a * b^T */
  m3 r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      r.m[i][j] = (a->m[i][0] * b->m[j][0] + a->m[i][1] * b->m[j][1]) + a->m[i][2] * b->m[j][2];
  return r;
}
static m3 m3_mul_at(const m3* a, const m3* b) { /* a^T * b */
  m3 r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      r.m[i][j] = (a->m[0][i] * b->m[0][j] + a->m[1][i] * b->m[1][j]) + a->m[2][i] * b->m[2][j];
  return r;
}
static m3 m3_identity(void) {
  m3 r;
  memset(&r, 0, sizeof r);
  r.m[0][0] = r.m[1][1] = r.m[2][2] = 1.0;
  return r;
}
/* MatrixBase::determinant for 3x3 (Eigen/src/LU/Determinant.h:18-23, 61-68). */
static double m3_det(const m3* a) {
  const double (*m)[3] = a->m;
  double h0 = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]);
  double h1 = m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]);
  double h2 = m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
  return (h0 - h1) + h2;
}
/* cofactor_3x3<i,j> (Eigen/src/LU/Inverse.h:117-127). */
static double cof(const m3* a, int i, int j) {
  int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
  return a->m[i1][j1] * a->m[i2][j2] - a->m[i1][j2] * a->m[i2][j1];
}
/* compute_inverse<...,3> (Eigen/src/LU/Inverse.h:130-158). */
static m3 m3_inverse(const m3* a) {
  double c0 = cof(a, 0, 0), c1 = cof(a, 1, 0), c2 = cof(a, 2, 0);
  double det = c0 * a->m[0][0] + (c1 * a->m[1][0] + c2 * a->m[2][0]);
  double invdet = 1.0 / det;
  m3 r;
  r.m[0][0] = c0 * invdet;
  r.m[0][1] = c1 * invdet;
  r.m[0][2] = c2 * invdet;
  r.m[1][0] = cof(a, 0, 1) * invdet;
  r.m[1][1] = cof(a, 1, 1) * invdet;
  r.m[1][2] = cof(a, 2, 1) * invdet;
  r.m[2][0] = cof(a, 0, 2) * invdet;
  r.m[2][1] = cof(a, 1, 2) * invdet;
  r.m[2][2] = cof(a, 2, 2) * invdet;
  return r;
}

/* Cyclic Jacobi eigen-decomposition of a symmetric 3x3 A = V diag(w) V^T,
 * w sorted decreasing (the singular values of the PSD F^T F). */
static void sym_eig3(const m3* A, double w[3], m3* V) {
  double a[3][3];
  memcpy(a, A->m, sizeof a);
  m3 v = m3_identity();
  for (int sweep = 0; sweep < 50; sweep++) {
    double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
    double scale = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]);
    if (off == 0.0 || off <= 1e-300 + 1e-18 * scale) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        double apq = a[p][q];
        if (apq == 0.0) continue;
        double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; k++) { /* A <- A J */
          double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; k++) { /* A <- J^T A */
          double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; k++) {
          double vkp = v.m[k][p], vkq = v.m[k][q];
          v.m[k][p] = c * vkp - s * vkq;
          v.m[k][q] = s * vkp + c * vkq;
        }
      }
  }
  int ord[3] = {0, 1, 2};
  double d[3] = {a[0][0], a[1][1], a[2][2]};
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (d[ord[j]] > d[ord[i]]) {
        int t = ord[i];
        ord[i] = ord[j];
        ord[j] = t;
      }
  for (int c = 0; c < 3; c++) {
    w[c] = d[ord[c]];
    if (w[c] < 0.0) w[c] = 0.0; /* singular values are >= 0 */
    for (int r = 0; r < 3; r++) V->m[r][c] = v.m[r][ord[c]];
  }
}

/* COROTATION (src/material/COROTATION.cpp) state for one F. */
typedef struct {
  double lambda, mu;
  m3 U, Fhat, V, R, S, L;
} corot;

/* COROTATION::orthogonalizeU (COROTATION.cpp:127-230). */
static void orthogonalize_u(m3* U, m3* Fhat) {
  double signU = (m3_det(U) >= 0.0) ? 1.0 : -1.0;
  const double small = 1e-4;
  int invalid[3] = {0, 0, 0}, total = 0;
  for (int x = 0; x < 3; x++)
    if (Fhat->m[x][x] < small) {
      invalid[x] = 1;
      total++;
    }
  if (total == 0) return;
  if (total == 1) {
    int w = 0;
    if (invalid[1]) w = 1;
    if (invalid[2]) w = 2;
    double c0[3], c1[3], c2[3];
    for (int r = 0; r < 3; r++) {
      c0[r] = U->m[r][(w + 1) % 3];
      c1[r] = U->m[r][(w + 2) % 3];
    }
    c2[0] = c0[1] * c1[2] - c0[2] * c1[1];
    c2[1] = c0[2] * c1[0] - c0[0] * c1[2];
    c2[2] = c0[0] * c1[1] - c0[1] * c1[0];
    double n = sqrt(c2[0] * c2[0] + (c2[1] * c2[1] + c2[2] * c2[2]));
    if (n > 0) for (int r = 0; r < 3; r++) c2[r] /= n;
    for (int r = 0; r < 3; r++) U->m[r][w] = c2[r];
    if (signU * m3_det(U) < 0.0)
      for (int r = 0; r < 3; r++) U->m[r][w] = -c2[r];
    return;
  } else if (total == 2) {
    int wv = 0;
    if (!invalid[1]) wv = 1;
    if (!invalid[2]) wv = 2;
    double v[3] = {U->m[0][wv], U->m[1][wv], U->m[2][wv]};
    int sm = (fabs(v[0]) < fabs(v[1])) ? 0 : 1;
    sm = (fabs(v[2]) < fabs(v[sm])) ? 2 : sm;
    double sv[3];
    int nx = (sm + 1) % 3, nn = (sm + 2) % 3;
    sv[sm] = 0.0;
    sv[nx] = -v[nn];
    sv[nn] = v[nx];
    double tv[3] = {v[1] * sv[2] - v[2] * sv[1], v[2] * sv[0] - v[0] * sv[2],
                    v[0] * sv[1] - v[1] * sv[0]};
    double n = sqrt(tv[0] * tv[0] + (tv[1] * tv[1] + tv[2] * tv[2]));
    if (n > 0) for (int r = 0; r < 3; r++) tv[r] /= n;
    nx = (wv + 1) % 3;
    nn = (wv + 2) % 3;
    for (int r = 0; r < 3; r++) {
      U->m[r][nx] = sv[r];
      U->m[r][nn] = tv[r];
    }
    if (signU * m3_det(U) < 0.0) {
      if (Fhat->m[nx][nx] < Fhat->m[nn][nn])
        for (int r = 0; r < 3; r++) U->m[r][nx] = -sv[r];
      else
        for (int r = 0; r < 3; r++) U->m[r][nn] = -tv[r];
    }
    return;
  }
  *U = m3_identity();
}

/* COROTATION::svd (COROTATION.cpp:235-280) + removeUReflection (:112-122). */
static void corot_svd(const m3* F, m3* U, m3* Fhat, m3* V) {
  m3 FtF = m3_mul_at(F, F);
  double w[3];
  sym_eig3(&FtF, w, V);
  memset(Fhat, 0, sizeof *Fhat);
  for (int i = 0; i < 3; i++) {
    Fhat->m[i][i] = sqrt(w[i]);
    if (isnan(Fhat->m[i][i])) Fhat->m[i][i] = 0.0;
  }
  if (m3_det(V) < 0.0)
    for (int r = 0; r < 3; r++) V->m[r][0] *= -1.0;
  m3 D;
  memset(&D, 0, sizeof D);
  for (int i = 0; i < 3; i++) D.m[i][i] = (Fhat->m[i][i] > 0.0) ? 1.0 / Fhat->m[i][i] : 0.0;
  m3 FV = m3_mul(F, V);
  *U = m3_mul(&FV, &D);
  orthogonalize_u(U, Fhat);
  if (m3_det(F) < 0.0) {
    int sm = (Fhat->m[0][0] < Fhat->m[1][1]) ? 0 : 1;
    sm = (Fhat->m[sm][sm] < Fhat->m[2][2]) ? sm : 2;
    Fhat->m[sm][sm] *= -1.0;
    for (int r = 0; r < 3; r++) U->m[r][sm] *= -1.0;
  }
}

/* COROTATION::init -> decomposeF (COROTATION.cpp:37-39, 91-107). */
static void corot_init(corot* c, const m3* F) {
  corot_svd(F, &c->U, &c->Fhat, &c->V);
  c->R = m3_mul_bt(&c->U, &c->V);
  m3 VF = m3_mul(&c->V, &c->Fhat);
  c->S = m3_mul_bt(&VF, &c->V);
  double trF = sum3(c->Fhat.m[0][0], c->Fhat.m[1][1], c->Fhat.m[2][2]);
  double trFm1 = sum3(c->Fhat.m[0][0] - 1.0, c->Fhat.m[1][1] - 1.0, c->Fhat.m[2][2] - 1.0);
  m3 T;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) T.m[i][j] = (i == j ? trF : 0.0) - c->Fhat.m[i][j];
  m3 Ti = m3_inverse(&T);
  double k = c->lambda * trFm1 - 2.0 * c->mu;
  m3 Ld;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Ld.m[i][j] = (i == j ? c->mu : 0.0) + k * Ti.m[i][j];
  for (int i = 0; i < 3; i++) Ld.m[i][i] = Ld.m[i][i] > 0 ? Ld.m[i][i] : 0;
  m3 VL = m3_mul(&c->V, &Ld);
  c->L = m3_mul_bt(&VL, &c->V);
}
/* COROTATION::strainEnergy (COROTATION.cpp:42-49). */
static double corot_energy(const corot* c) {
  m3 E = c->S;
  for (int i = 0; i < 3; i++) E.m[i][i] -= 1.0;
  m3 EtE = m3_mul_at(&E, &E);
  double tr = sum3(EtE.m[0][0], EtE.m[1][1], EtE.m[2][2]);
  double trE = sum3(E.m[0][0], E.m[1][1], E.m[2][2]);
  return c->mu * tr + 0.5 * c->lambda * (trE * trE);
}
/* COROTATION::firstPiolaKirchhoff (COROTATION.cpp:53-62). */
static m3 corot_pk1(const corot* c) {
  m3 E = c->S;
  for (int i = 0; i < 3; i++) E.m[i][i] -= 1.0;
  m3 t;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) t.m[i][j] = 2.0 * c->mu * E.m[i][j];
  double tr = c->lambda * sum3(E.m[0][0], E.m[1][1], E.m[2][2]);
  for (int i = 0; i < 3; i++) t.m[i][i] += tr;
  return m3_mul(&c->R, &t);
}
/* COROTATION::firstPKDifferential (COROTATION.cpp:64-84), including its
 * second lambda*tr(dFhat) on the diagonal. */
static m3 corot_dpk(const corot* c, const m3* dF) {
  m3 dFhat = m3_mul_at(&c->R, dF);
  m3 sym, skew;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      sym.m[i][j] = 0.5 * (dFhat.m[i][j] + dFhat.m[j][i]);
      skew.m[i][j] = 0.5 * (dFhat.m[i][j] - dFhat.m[j][i]);
    }
  double trs = sum3(sym.m[0][0], sym.m[1][1], sym.m[2][2]);
  m3 dP;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      dP.m[i][j] = (2.0 * c->mu * sym.m[i][j]) + (i == j ? c->lambda * trs : 0.0);
  double f[3] = {-skew.m[1][2] + skew.m[2][1], -skew.m[2][0] + skew.m[0][2],
                 -skew.m[0][1] + skew.m[1][0]};
  double tr = c->lambda * sum3(dFhat.m[0][0], dFhat.m[1][1], dFhat.m[2][2]);
  for (int i = 0; i < 3; i++) dP.m[i][i] += tr;
  double Lf[3];
  for (int i = 0; i < 3; i++) Lf[i] = (c->L.m[i][0] * f[0] + c->L.m[i][1] * f[1]) + c->L.m[i][2] * f[2];
  /* MATRIX_UTIL::cross(v) (include/linearalgebra/MATRIX_UTIL.h:26-41) */
  dP.m[0][1] += -Lf[2];
  dP.m[0][2] += Lf[1];
  dP.m[1][0] += Lf[2];
  dP.m[1][2] += -Lf[0];
  dP.m[2][0] += -Lf[1];
  dP.m[2][1] += Lf[0];
  return m3_mul(&c->R, &dP);
}

/* --------------------------------------------------------------- state --- */
typedef struct {
  /* static description */
  int mres[3];
  double mdh, morig[3];
  double* rest; /* rest mass grid */
  double lambda, mu, qcm; /* _quarterCellSolidMass = rho dh^3 / 8 */
  double rot[9], trans[3], scale[3], v0[3];
  int nv, ntri;
  double *restPose, *verts;
  int* tris;
  /* fields (node-indexed) */
  double *X, *u, *vel, *vws, *mass, *phi, *detFInv, *quarter, *tmp3;
  signed char* valid; /* (X-1)(Y-1)(Z-1) */
  int xmin, ymin, zmin, xmax, ymax, zmax;
  int tmin[3], tmax[3];
  double dt;
  long np, pcap;
  double* part; /* 10 per particle: pos, vel, rest, mass */
  double safeMin[3], safeMax[3];
  double G[8][3];
  /* plasticity (setPlasticYield, DEFOR_SOLID_3D.h:55-58; material grid of
   * loadSurfaceMesh, DEFOR_SOLID_3D.cpp:175-186) */
  int plastic;
  double yield;
  int pres[3];
  double pdh, porig[3];
  double *FpInv, *FpNew; /* 9 per material cell, row-major */
  double pgrid[7];       /* xRes, yRes, zRes, dh, origin */
  signed char* fpSet;
} solid_t;

struct esfo_scene {
  esf_grid g;
  esf_params p;
  int X, Y, Z, slab, total, cells, nInterior, nSolid;
  double dh, dhInv, o[3];
  int ns;
  solid_t* s[MAXS];
  int inited;
  double fluidDensity, defaultDt, dt, vortEps;
  /* node fields */
  double *vel, *vws, *vort, *intensity, *ws, *solidMass, *nodeVF, *quarter;
  int *dof, *sdof;
  /* vectors */
  double *unitForce, *mv, *nzMassInv, *vstar, *v1, *pc; /* D */
  double *solidUnitForce, *solidMv, *damped, *solidV0, *solidPC, *solidB1, *sysDiag; /* 3S */
  double *jdiag, *rhs, *b1, *lambda; /* R */
  int haveLambda;
  /* system matrix CSR (3S rows) */
  int *Ap, *Aj;
  double* Ax;
  long annz;
  /* scratch */
  double *tA, *tB, *tC, *tD, *tE, *tF, *tG, *mid;
  int status;
};

#define NIDX(x, y, z) ((x) + (y) * s->X + (z) * s->slab)

static void* xcalloc(size_t n, size_t sz) {
  void* p = calloc(n ? n : 1, sz);
  if (!p) {
    fprintf(stderr, "esf_oracle: out of memory (%zu x %zu)\n", n, sz);
    abort();
  }
  return p;
}

int esfo_params_default(const esf_grid* g, esf_params* p) {
  if (!g || !p) return ESF_ERR_INVALID_ARG;
  memset(p, 0, sizeof *p);
  p->dt = 0.01;
  p->fluid_density = 1.0;
  p->fluid_viscosity = 0.0;
  p->vorticity_eps = 2.0;
  p->buoyancy = 0.1;
  p->gravity = 0.0;
  p->implicit_solver_eps = 1e-8;
  p->div_free_solver_eps = 1e-8;
  p->cr_max_iterations = 10;
  p->mass_sample_dh = g->dh / 10;
  p->tight_border = 3;
  p->extrapolation_cells = 20;
  p->particles_per_cell = 8;
  p->flip_alpha = 0.95;
  p->contact_safe_distance = g->dh * 0.5;
  p->wall_thickness = g->dh * 1.5;
  p->contact_spring_stiffness = 10000;
  p->friction = 0.5;
  p->flip_cutoff = 3;
  p->flow_rate = 0.0;
  p->precision = ESF_FP64;
  p->inner_eps = 1e-4;
  p->max_refinements = 50;
  return ESF_OK;
}

/* COUPLED_INTEGRATOR_3D::COUPLED_INTEGRATOR_3D (COUPLED_INTEGRATOR_3D.cpp:36-78). */
esfo_scene* esfo_create(const esf_grid* g, const esf_params* p) {
  if (!g || !p || g->xRes < 4 || g->yRes < 4 || g->zRes < 4 || !(g->dh > 0)) return NULL;
  esfo_scene* s = (esfo_scene*)xcalloc(1, sizeof *s);
  s->g = *g;
  s->p = *p;
  s->X = g->xRes;
  s->Y = g->yRes;
  s->Z = g->zRes;
  s->slab = s->X * s->Y;
  s->total = s->slab * s->Z;
  s->cells = (s->X - 1) * (s->Y - 1) * (s->Z - 1);
  s->nInterior = (s->X - 2) * (s->Y - 2) * (s->Z - 2);
  s->dh = g->dh;
  s->dhInv = 1.0 / g->dh;
  for (int k = 0; k < 3; k++) s->o[k] = g->origin[k];
  s->fluidDensity = 1.0;
  s->defaultDt = p->dt;
  s->dt = p->dt;
  int maxRes = imax(imax(s->X, s->Y), s->Z);
  double scaling = 64.0f / maxRes;
  scaling = (scaling < 1.0f) ? 1.0f : scaling;
  s->vortEps = p->vorticity_eps / scaling;
  long T = s->total;
  s->vel = xcalloc(T * 3, 8);
  s->vws = xcalloc(T * 3, 8);
  s->vort = xcalloc(T * 3, 8);
  s->intensity = xcalloc(T, 8);
  s->ws = xcalloc(T, 8);
  s->solidMass = xcalloc(T, 8);
  s->nodeVF = xcalloc(T, 8);
  s->quarter = xcalloc(T * 8, 8);
  s->dof = xcalloc(T, 4);
  s->sdof = xcalloc(T, 4);
  for (long i = 0; i < T; i++) s->dof[i] = s->sdof[i] = -1;
  long D = 3L * s->nInterior, R = s->cells;
  s->unitForce = xcalloc(D, 8);
  s->mv = xcalloc(D, 8);
  s->nzMassInv = xcalloc(D, 8);
  s->vstar = xcalloc(D, 8);
  s->v1 = xcalloc(D, 8);
  s->pc = xcalloc(D, 8);
  s->mid = xcalloc(D, 8);
  s->jdiag = xcalloc(R, 8);
  s->rhs = xcalloc(R, 8);
  s->b1 = xcalloc(R, 8);
  s->lambda = xcalloc(R, 8);
  long W = (D > R ? D : R);
  s->tA = xcalloc(W, 8);
  s->tB = xcalloc(W, 8);
  s->tC = xcalloc(W, 8);
  s->tD = xcalloc(W, 8);
  s->tE = xcalloc(W, 8);
  s->tF = xcalloc(W, 8);
  s->tG = xcalloc(W, 8);
  return s;
}

static void free_solid(solid_t* d) {
  if (!d) return;
  free(d->rest); free(d->restPose); free(d->verts); free(d->tris);
  free(d->X); free(d->u); free(d->vel); free(d->vws); free(d->mass); free(d->phi);
  free(d->detFInv); free(d->quarter); free(d->tmp3); free(d->valid); free(d->part);
  free(d->FpInv); free(d->FpNew); free(d->fpSet);
  free(d);
}

static void free_solid_vectors(esfo_scene* s) {
  free(s->solidUnitForce); free(s->solidMv); free(s->damped); free(s->solidV0);
  free(s->solidPC); free(s->solidB1); free(s->sysDiag);
  s->solidUnitForce = s->solidMv = s->damped = s->solidV0 = s->solidPC = s->solidB1 = s->sysDiag = NULL;
}

void esfo_destroy(esfo_scene* s) {
  if (!s) return;
  for (int i = 0; i < s->ns; i++) free_solid(s->s[i]);
  free(s->vel); free(s->vws); free(s->vort); free(s->intensity); free(s->ws);
  free(s->solidMass); free(s->nodeVF); free(s->quarter); free(s->dof); free(s->sdof);
  free(s->unitForce); free(s->mv); free(s->nzMassInv); free(s->vstar); free(s->v1); free(s->pc);
  free(s->mid); free(s->jdiag); free(s->rhs); free(s->b1); free(s->lambda);
  free(s->tA); free(s->tB); free(s->tC); free(s->tD); free(s->tE); free(s->tF); free(s->tG);
  free_solid_vectors(s);
  free(s->Ap); free(s->Aj); free(s->Ax);
  free(s);
}

int esfo_set_fluid(esfo_scene* s, double density, double viscosity) {
  if (!s) return ESF_ERR_INVALID_ARG;
  (void)viscosity; /* stored but never used by the reference (:46) */
  s->fluidDensity = density;
  return ESF_OK;
}
int esfo_set_max_dt(esfo_scene* s, double max_dt) {
  if (!s) return ESF_ERR_INVALID_ARG;
  s->defaultDt = max_dt;
  return ESF_OK;
}
double esfo_dt(const esfo_scene* s) { return s ? s->dt : 0.0; }

/* -------------------------------------------------------- interpolation -- */
/* FIELD_3D::get_barycentric (FIELD_3D.h:368-382). */
static inline void bary(double x, double dh, int* i, double* f, int ihigh) {
  x /= dh;
  double sfl = floor(x);
  int ii = (int)sfl;
  if (ii < 0) {
    *i = 0;
    *f = 0.5;
  } else if (ii > ihigh) {
    *i = ihigh;
    *f = 0.5;
  } else {
    *i = ii;
    *f = x - sfl;
  }
}
static inline double lerp(double a, double b, double f) { return (1 - f) * a + f * b; }
/* FIELD_3D::interpolate_value (FIELD_3D.h:198-216), trilerp order of
 * MATH_UTILS.h:325-342. */
static double interp1(const double* d, int X, int Y, int Z, double dh, const double* o,
                      const double* p) {
  int i, j, k;
  double fx, fy, fz;
  bary(p[0] - o[0], dh, &i, &fx, X - 2);
  bary(p[1] - o[1], dh, &j, &fy, Y - 2);
  bary(p[2] - o[2], dh, &k, &fz, Z - 2);
  long sl = (long)X * Y;
  long b = i + (long)j * X + k * sl;
  double v000 = d[b], v100 = d[b + 1], v010 = d[b + X], v110 = d[b + X + 1];
  double v001 = d[b + sl], v101 = d[b + sl + 1], v011 = d[b + sl + X], v111 = d[b + sl + X + 1];
  double a0 = lerp(lerp(v000, v100, fx), lerp(v010, v110, fx), fy);
  double a1 = lerp(lerp(v001, v101, fx), lerp(v011, v111, fx), fy);
  return lerp(a0, a1, fz);
}
/* VEC3F_FIELD_3D::interpolate_value (VEC3F_FIELD_3D.h:179-197). */
static void interp3(const double* d, int X, int Y, int Z, double dh, const double* o,
                    const double* p, double* out) {
  int i, j, k;
  double fx, fy, fz;
  bary(p[0] - o[0], dh, &i, &fx, X - 2);
  bary(p[1] - o[1], dh, &j, &fy, Y - 2);
  bary(p[2] - o[2], dh, &k, &fz, Z - 2);
  long sl = (long)X * Y;
  long b = i + (long)j * X + k * sl;
  for (int c = 0; c < 3; c++) {
    double v000 = d[3 * b + c], v100 = d[3 * (b + 1) + c], v010 = d[3 * (b + X) + c],
           v110 = d[3 * (b + X + 1) + c];
    double v001 = d[3 * (b + sl) + c], v101 = d[3 * (b + sl + 1) + c],
           v011 = d[3 * (b + sl + X) + c], v111 = d[3 * (b + sl + X + 1) + c];
    double a0 = lerp(lerp(v000, v100, fx), lerp(v010, v110, fx), fy);
    double a1 = lerp(lerp(v001, v101, fx), lerp(v011, v111, fx), fy);
    out[c] = lerp(a0, a1, fz);
  }
}
#define I1(S, field, p) interp1((field), (S)->X, (S)->Y, (S)->Z, (S)->dh, (S)->o, (p))
#define I3(S, field, p, out) interp3((field), (S)->X, (S)->Y, (S)->Z, (S)->dh, (S)->o, (p), (out))

/* -------------------------------------------------------------- solids --- */
/* DEFOR_SOLID_3D ctor + setters + setInitialState + loadSurfaceMesh
 * (DEFOR_SOLID_3D.cpp:43-84, 113-207; main.cpp:99-160). */
int esfo_add_solid(esfo_scene* s, const esf_solid_desc* dd) {
  if (!s || !dd || s->inited || s->ns >= MAXS) return ESF_ERR_INVALID_ARG;
  if (!dd->rest_mass || dd->mass_res[0] < 2 || dd->mass_res[1] < 2 || dd->mass_res[2] < 2)
    return ESF_ERR_INVALID_ARG;
  if (dd->num_vertices <= 0 || !dd->vertices || dd->num_triangles <= 0 || !dd->triangles)
    return ESF_ERR_INVALID_ARG;
  solid_t* d = (solid_t*)xcalloc(1, sizeof *d);
  long T = s->total;
  for (int k = 0; k < 3; k++) {
    d->mres[k] = dd->mass_res[k];
    d->morig[k] = dd->mass_origin[k];
    d->trans[k] = dd->translation[k];
    d->scale[k] = dd->scaling[k];
    d->v0[k] = dd->initial_velocity[k];
  }
  d->mdh = dd->mass_dh;
  long mn = (long)d->mres[0] * d->mres[1] * d->mres[2];
  d->rest = xcalloc(mn, 8);
  memcpy(d->rest, dd->rest_mass, mn * 8);
  memcpy(d->rot, dd->rotation, sizeof d->rot);
  d->lambda = dd->lambda;
  d->mu = dd->mu;
  d->qcm = dd->density * s->dh * s->dh * s->dh * 0.125; /* setMassDensity (DEFOR_SOLID_3D.h:64-66) */
  d->X = xcalloc(T * 3, 8);
  d->u = xcalloc(T * 3, 8);
  d->vel = xcalloc(T * 3, 8);
  d->vws = xcalloc(T * 3, 8);
  d->tmp3 = xcalloc(T * 3, 8);
  d->mass = xcalloc(T, 8);
  d->phi = xcalloc(T, 8);
  d->detFInv = xcalloc(T, 8);
  d->quarter = xcalloc(T * 8, 8);
  d->valid = xcalloc(s->cells, 1);
  d->dt = s->p.dt;
  for (int k = 0; k < 3; k++) {
    d->safeMin[k] = s->o[k] + 2 * s->dh;
  }
  d->safeMax[0] = s->o[0] + (s->X - 3) * s->dh;
  d->safeMax[1] = s->o[1] + (s->Y - 3) * s->dh;
  d->safeMax[2] = s->o[2] + (s->Z - 3) * s->dh;
  /* setInitialState (DEFOR_SOLID_3D.cpp:126-152): X = R^T (x - T) / s. */
  for (int z = 0; z < s->Z; z++)
    for (int y = 0; y < s->Y; y++)
      for (int x = 0; x < s->X; x++) {
        long n = NIDX(x, y, z);
        double pt[3] = {(double)x, (double)y, (double)z};
        for (int k = 0; k < 3; k++) {
          pt[k] *= s->dh;
          pt[k] += s->o[k];
          pt[k] -= d->trans[k];
        }
        double q[3];
        for (int i = 0; i < 3; i++) /* rotation.transpose() * point */
          q[i] = (d->rot[0 * 3 + i] * pt[0] + d->rot[1 * 3 + i] * pt[1]) + d->rot[2 * 3 + i] * pt[2];
        for (int k = 0; k < 3; k++) d->X[3 * n + k] = q[k] / d->scale[k];
      }
  for (int z = 0; z < s->Z; z++)
    for (int y = 0; y < s->Y; y++)
      for (int x = 0; x < s->X; x++) {
        long n = NIDX(x, y, z);
        double pos[3] = {x * s->dh, y * s->dh, z * s->dh};
        for (int k = 0; k < 3; k++) {
          pos[k] += s->o[k];
          d->u[3 * n + k] = pos[k] - d->X[3 * n + k];
        }
      }
  /* setInitialVelocity (:153-155) */
  for (long i = 0; i < T; i++)
    for (int k = 0; k < 3; k++) d->vel[3 * i + k] = d->v0[k];
  /* mesh: rest pose kept; current pose = scale, rotate, translate
   * (OBJ::scale / transformMesh / translateMesh, main.cpp:150-154). */
  d->nv = dd->num_vertices;
  d->ntri = dd->num_triangles;
  d->restPose = xcalloc(d->nv * 3, 8);
  d->verts = xcalloc(d->nv * 3, 8);
  d->tris = xcalloc(d->ntri * 3, 4);
  memcpy(d->restPose, dd->vertices, d->nv * 24);
  memcpy(d->tris, dd->triangles, d->ntri * 12);
  for (int t = 0; t < d->ntri * 3; t++)
    if (d->tris[t] < 0 || d->tris[t] >= d->nv) {
      free_solid(d);
      return ESF_ERR_INVALID_ARG;
    }
  for (int v = 0; v < d->nv; v++) {
    double p[3];
    for (int k = 0; k < 3; k++) p[k] = d->restPose[3 * v + k] * d->scale[k];
    double q[3];
    for (int i = 0; i < 3; i++)
      q[i] = (d->rot[i * 3 + 0] * p[0] + d->rot[i * 3 + 1] * p[1]) + d->rot[i * 3 + 2] * p[2];
    for (int k = 0; k < 3; k++) d->verts[3 * v + k] = q[k] + d->trans[k];
  }
  /* the inverse plastic deformation gradient lives on a grid of half the
   * cell size over the rest mesh's box grown by one cell
   * (DEFOR_SOLID_3D.cpp:158-186), identity at the start */
  if (dd->plastic_yield > 0) {
    d->plastic = 1;
    d->yield = dd->plastic_yield;
    double bmin[3] = {1e9, 1e9, 1e9}, bmax[3] = {-1e9, -1e9, -1e9};
    for (int v = 0; v < d->nv; v++)
      for (int k = 0; k < 3; k++) {
        bmin[k] = fmin(bmin[k], d->restPose[3 * v + k]);
        bmax[k] = fmax(bmax[k], d->restPose[3 * v + k]);
      }
    d->pdh = s->dh * .5;
    for (int k = 0; k < 3; k++) {
      bmin[k] -= s->dh;
      bmax[k] += s->dh;
      d->pres[k] = (int)((bmax[k] - bmin[k]) / d->pdh + 1);
      d->porig[k] = bmin[k];
    }
    long pn = (long)d->pres[0] * d->pres[1] * d->pres[2];
    d->FpInv = xcalloc(pn * 9, 8);
    d->FpNew = xcalloc(pn * 9, 8);
    d->fpSet = xcalloc(pn, 1);
    for (long c = 0; c < pn; c++)
      for (int i = 0; i < 3; i++) d->FpInv[c * 9 + i * 4] = 1.0;
    double hdr[7] = {d->pres[0], d->pres[1], d->pres[2], d->pdh, d->porig[0], d->porig[1], d->porig[2]};
    memcpy(d->pgrid, hdr, sizeof hdr);
  }
  /* _G (DEFOR_SOLID_3D.cpp:304-310) */
  for (int i = 0; i < 8; i++) {
    d->G[i][0] = (i % 2 == 0 ? -1 : 1) * (0.25 * s->dhInv);
    d->G[i][1] = (i % 4 <= 1 ? -1 : 1) * (0.25 * s->dhInv);
    d->G[i][2] = (i < 4 ? -1 : 1) * (0.25 * s->dhInv);
  }
  s->s[s->ns++] = d;
  return ESF_OK;
}

/* DEFOR_SOLID_3D::computeF (DEFOR_SOLID_3D.cpp:671-682): returns det F
 * (or 1 when |det F^-1| <= 1e-4, with F = I). corner[i] = u at corner i. */
static double compute_F(const solid_t* d, const double corner[8][3], m3* F) {
  m3 Finv;
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      double acc = corner[0][r] * d->G[0][c];
      for (int k = 1; k < 8; k++) acc += corner[k][r] * d->G[k][c];
      Finv.m[r][c] = (r == c ? 1.0 : 0.0) - acc;
    }
  double Jinv = m3_det(&Finv);
  if (fabs(Jinv) > 1e-4) {
    *F = m3_inverse(&Finv);
  } else {
    *F = m3_identity();
    Jinv = 1;
  }
  return 1.0 / Jinv;
}

static void gather_corners(const esfo_scene* s, const double* f, long index, double c[8][3]) {
  const long off[8] = {0, 1, s->X, s->X + 1, s->slab, s->slab + 1, s->slab + s->X,
                       s->slab + s->X + 1};
  for (int i = 0; i < 8; i++)
    for (int k = 0; k < 3; k++) c[i][k] = f[3 * (index + off[i]) + k];
}

#define VIDX(x, y, z) ((x) + (y) * (s->X - 1) + (z) * (s->X - 1) * (s->Y - 1))

/* DEFOR_SOLID_3D::computeSolidMass (DEFOR_SOLID_3D.cpp:576-669). */
static void compute_solid_mass(esfo_scene* s, solid_t* d, int usesdf) {
  long T = s->total;
  memset(d->mass, 0, T * 8);
  memset(d->valid, 0, s->cells);
  memset(d->detFInv, 0, T * 8);
  memset(d->quarter, 0, T * 8 * 8);
  const double subDh = s->p.mass_sample_dh;
  const double subVol = subDh * subDh * subDh;
  const int res = (int)(s->dh / subDh);
  const int half = res >> 1;
  const double fraction = 1.0 / (res * res * res);
  const long off[8] = {0, 1, s->X, s->X + 1, s->slab, s->slab + 1, s->slab + s->X,
                       s->slab + s->X + 1};
  for (int z = d->tmin[2]; z < d->tmax[2] - 1; z++)
    for (int y = d->tmin[1]; y < d->tmax[1] - 1; y++)
      for (int x = d->tmin[0]; x < d->tmax[0] - 1; x++) {
        long index = NIDX(x, y, z);
        double c[8][3];
        gather_corners(s, d->u, index, c);
        m3 F;
        d->detFInv[index] = fabs(1.0 / compute_F(d, c, &F));
      }
  for (int z = d->tmin[2]; z < d->tmax[2] - 1; z++)
    for (int y = d->tmin[1]; y < d->tmax[1] - 1; y++)
      for (int x = d->tmin[0]; x < d->tmax[0] - 1; x++) {
        long index = NIDX(x, y, z);
        double node[3] = {x * s->dh + s->o[0], y * s->dh + s->o[1], z * s->dh + s->o[2]};
        if (usesdf && d->phi[index] > 2) continue;
        double* q = d->quarter + index * 8;
        for (int p = 0; p < res; p++)
          for (int qq = 0; qq < res; qq++)
            for (int r = 0; r < res; r++) {
              double pos[3] = {node[0] + (p + 0.5) * subDh, node[1] + (qq + 0.5) * subDh,
                               node[2] + (r + 0.5) * subDh};
              double rp[3];
              I3(s, d->X, pos, rp);
              double dd = interp1(d->rest, d->mres[0], d->mres[1], d->mres[2], d->mdh, d->morig, rp) * subVol;
              if (dd < 1e-6) continue;
              int o = p < half ? 0 : 1;
              o += qq < half ? 0 : 2;
              o += r < half ? 0 : 4;
              q[o] += fraction;
            }
        double sum = 0;
        for (int i = 0; i < 8; i++) sum += q[i];
        if (sum > 0.5) {
          for (int i = 0; i < 8; i++) q[i] = 1;
          d->valid[VIDX(x, y, z)] = 1;
        } else {
          if (sum > 0) d->valid[VIDX(x, y, z)] = 2;
          for (int i = 0; i < 8; i++) q[i] = 0;
        }
      }
  for (int i = 0; i < 8; i++)
    for (int z = d->tmin[2]; z < d->tmax[2] - 1; z++)
      for (int y = d->tmin[1]; y < d->tmax[1] - 1; y++)
        for (int x = d->tmin[0]; x < d->tmax[0] - 1; x++) {
          if (!d->valid[VIDX(x, y, z)]) continue;
          long index = NIDX(x, y, z);
          d->mass[index + off[i]] += d->quarter[index * 8 + i] * d->detFInv[index] * d->qcm;
        }
}

/* solveDistance (DEFOR_SOLID_3D.cpp:369-394). */
static void solve_distance(double p, double q, double r, double* v) {
  double ds[3];
  ds[0] = dmin(p, dmin(q, r));
  ds[2] = dmax(p, dmax(q, r));
  ds[1] = p + q + r - ds[0] - ds[2];
  double b[3], c[3];
  b[0] = ds[0];
  c[0] = ds[0] * ds[0] - 1.0f;
  for (int x = 1; x < 3; x++) {
    b[x] = ds[x] + b[x - 1];
    c[x] = ds[x] * ds[x] + c[x - 1];
  }
  int i = 2;
  double discrim = b[i] * b[i] - (double)(i + 1) * c[i];
  double newDist = (b[i] + sqrt(discrim)) / (double)(i + 1);
  while ((discrim < 0.0f || newDist < ds[i]) && i != -1) {
    i--;
    /* the reference reads b[-1]/c[-1] here when i reaches -1; that value
     * is never used because the loop then exits with newDist unchanged */
    if (i < 0) break;
    discrim = b[i] * b[i] - (double)(i + 1) * c[i];
    if (discrim > 0.0f) newDist = (b[i] + sqrt(discrim)) / (double)(i + 1);
  }
  if (newDist < *v) *v = newDist;
}

/* DEFOR_SOLID_3D::sweepPhi (DEFOR_SOLID_3D.cpp:397-455). */
static void sweep_phi(esfo_scene* s, solid_t* d) {
  double* ph = d->phi;
  const double* m = d->mass;
  const int X = s->X;
  const long sl = s->slab;
#define PH(i, j, k) ph[(i) + (long)(j) * X + (long)(k) * sl]
#define MS(i, j, k) m[(i) + (long)(j) * X + (long)(k) * sl]
  for (int dir = 0; dir < 8; dir++) {
    int dj = (dir & 1) ? -1 : 1; /* order of the 8 loops in the reference */
    int di = (dir & 2) ? -1 : 1;
    int dk = (dir & 4) ? -1 : 1;
    int k0 = dk > 0 ? d->zmin + 1 : d->zmax - 2, k1 = dk > 0 ? d->zmax : d->zmin - 1;
    int j0 = dj > 0 ? d->ymin + 1 : d->ymax - 2, j1 = dj > 0 ? d->ymax : d->ymin - 1;
    int i0 = di > 0 ? d->xmin + 1 : d->xmax - 2, i1 = di > 0 ? d->xmax : d->xmin - 1;
    for (int k = k0; k != k1; k += dk)
      for (int j = j0; j != j1; j += dj)
        for (int i = i0; i != i1; i += di)
          if (MS(i, j, k) == 0)
            solve_distance(PH(i - di, j, k), PH(i, j - dj, k), PH(i, j, k - dk), &PH(i, j, k));
  }
#undef PH
#undef MS
}

/* DEFOR_SOLID_3D::computeSDF (DEFOR_SOLID_3D.cpp:216-268). */
static void compute_sdf(esfo_scene* s, solid_t* d) {
  double large = s->X + s->Y + s->Z + 2;
  d->xmax = d->ymax = d->zmax = 0;
  d->xmin = s->X;
  d->ymin = s->Y;
  d->zmin = s->Z;
  long index = 0;
  for (int z = 0; z < s->Z; z++)
    for (int y = 0; y < s->Y; y++)
      for (int x = 0; x < s->X; x++, index++) {
        d->phi[index] = large;
        if (d->mass[index] > 0) {
          d->phi[index] = -0.5;
          if (x < d->xmin) d->xmin = x;
          if (x > d->xmax) d->xmax = x;
          if (y < d->ymin) d->ymin = y;
          if (y > d->ymax) d->ymax = y;
          if (z < d->zmin) d->zmin = z;
          if (z > d->zmax) d->zmax = z;
        }
      }
  int tb = s->p.tight_border, ex = s->p.extrapolation_cells;
  d->tmin[0] = imax(d->xmin - tb, 0);
  d->tmin[1] = imax(d->ymin - tb, 0);
  d->tmin[2] = imax(d->zmin - tb, 0);
  d->tmax[0] = imin(d->xmax + tb, s->X);
  d->tmax[1] = imin(d->ymax + tb, s->Y);
  d->tmax[2] = imin(d->zmax + tb, s->Z);
  d->xmin = imax(d->xmin - ex, 0);
  d->ymin = imax(d->ymin - ex, 0);
  d->zmin = imax(d->zmin - ex, 0);
  d->xmax = imin(d->xmax + ex, s->X);
  d->ymax = imin(d->ymax + ex, s->Y);
  d->zmax = imin(d->zmax + ex, s->Z);
  for (int i = 0; i < 2; ++i) sweep_phi(s, d);
}

/* DEFOR_SOLID_3D::initMaterialParticles (DEFOR_SOLID_3D.cpp:333-367).
 * The three rand() calls of VEC3F(rand, rand, rand) are consumed in the
 * order the reference's x86-64 g++ build evaluates them (z, y, x). */
static void init_particles(esfo_scene* s, solid_t* d) {
  const int ppc = s->p.particles_per_cell;
  const double density = d->qcm / (s->dh * s->dh * s->dh * 0.125);
  const double volume = s->dh * s->dh * s->dh / ppc;
  mt19937 tw;
  mt_seed(&tw, 123456u);
  long n = 0;
  for (int z = d->tmin[2]; z < d->tmax[2] - 1; z++)
    for (int y = d->tmin[1]; y < d->tmax[1] - 1; y++)
      for (int x = d->tmin[0]; x < d->tmax[0] - 1; x++)
        if (d->valid[VIDX(x, y, z)] == 1) n += ppc;
  if (n > d->pcap) {
    free(d->part);
    d->part = xcalloc(n * 10, 8);
    d->pcap = n;
  }
  d->np = n;
  long c = 0;
  for (int z = d->tmin[2]; z < d->tmax[2] - 1; z++)
    for (int y = d->tmin[1]; y < d->tmax[1] - 1; y++)
      for (int x = d->tmin[0]; x < d->tmax[0] - 1; x++) {
        if (d->valid[VIDX(x, y, z)] != 1) continue;
        double grid[3] = {s->o[0] + x * s->dh, s->o[1] + y * s->dh, s->o[2] + z * s->dh};
        for (int i = 0; i < ppc; i++, c++) {
          double r2 = mt_rand(&tw, s->dh);
          double r1 = mt_rand(&tw, s->dh);
          double r0 = mt_rand(&tw, s->dh);
          double* P = d->part + c * 10;
          P[0] = grid[0] + r0;
          P[1] = grid[1] + r1;
          P[2] = grid[2] + r2;
          I3(s, d->X, P, P + 6);
          I3(s, d->vel, P, P + 3);
          P[9] = density * volume;
        }
      }
}

/* DEFOR_SOLID_3D::advectSurfaceMesh (DEFOR_SOLID_3D.cpp:1125-1180). */
static void advect_mesh(esfo_scene* s, solid_t* d) {
  const double eps = 1e-4;
  for (int v = 0; v < d->nv; v++) {
    double* vx = d->verts + 3 * v;
    double vel[3];
    I3(s, d->vel, vx, vel);
    for (int k = 0; k < 3; k++) vx[k] += vel[k] * d->dt;
    double residual = 1;
    int count = 0;
    while (residual > eps && count++ < 10) {
      double uu[3], diff[3];
      I3(s, d->u, vx, uu);
      for (int k = 0; k < 3; k++) diff[k] = (vx[k] - uu[k]) - d->restPose[3 * v + k];
      residual = sqrt(diff[0] * diff[0] + (diff[1] * diff[1] + diff[2] * diff[2]));
      int i = (int)((vx[0] - s->o[0]) / s->dh);
      if (i < 0) i = 0;
      if (i > s->X - 2) i = s->X - 2;
      int j = (int)((vx[1] - s->o[1]) / s->dh);
      if (j < 0) j = 0;
      if (j > s->Y - 2) j = s->Y - 2;
      int k = (int)((vx[2] - s->o[2]) / s->dh);
      if (k < 0) k = 0;
      if (k > s->Z - 2) k = s->Z - 2;
      double c[8][3];
      gather_corners(s, d->u, NIDX(i, j, k), c);
      m3 F;
      compute_F(d, c, &F);
      for (int r = 0; r < 3; r++)
        vx[r] -= (F.m[r][0] * diff[0] + F.m[r][1] * diff[1]) + F.m[r][2] * diff[2];
    }
    vx[0] = dmax(s->o[0], vx[0]);
    vx[1] = dmax(s->o[1], vx[1]);
    vx[2] = dmax(s->o[2], vx[2]);
    vx[0] = dmin(s->o[0] + s->dh * (s->X - 1), vx[0]);
    vx[1] = dmin(s->o[1] + s->dh * (s->Y - 1), vx[1]);
    vx[2] = dmin(s->o[2] + s->dh * (s->Z - 1), vx[2]);
  }
}

/* DEFOR_SOLID_3D::recoverVelocityField (DEFOR_SOLID_3D.cpp:1235-1241). */
static void recover_velocity(esfo_scene* s, solid_t* d, double* v) {
  for (int z = d->zmin; z < d->zmax - 1; z++)
    for (int y = d->ymin; y < d->ymax - 1; y++)
      for (int x = d->xmin; x < d->xmax - 1; x++) {
        long n = NIDX(x, y, z);
        if (d->mass[n] > 0)
          for (int k = 0; k < 3; k++) v[3 * n + k] = d->vel[3 * n + k];
      }
}

/* COUPLED_INTEGRATOR_3D::gatherSolidMasses (COUPLED_INTEGRATOR_3D.cpp:327-375). */
static void gather_solid_masses(esfo_scene* s) {
  long T = s->total;
  memset(s->solidMass, 0, T * 8);
  memset(s->quarter, 0, T * 64);
  for (int i = 0; i < s->ns; i++)
    for (long n = 0; n < T; n++) s->solidMass[n] += s->s[i]->mass[n];
  for (int i = 0; i < s->ns; i++)
    for (long n = 0; n < T * 8; n++) s->quarter[n] += s->s[i]->quarter[n];
  memset(s->nodeVF, 0, T * 8);
  const long off[8] = {0, 1, s->X, s->X + 1, s->slab, s->slab + 1, s->slab + s->X,
                       s->slab + s->X + 1};
  for (int i = 0; i < 8; i++)
    for (int z = 1; z < s->Z - 1; z++)
      for (int y = 1; y < s->Y - 1; y++)
        for (int x = 1; x < s->X - 1; x++) {
          long index = NIDX(x, y, z);
          s->nodeVF[index + off[i]] += s->quarter[index * 8 + i];
        }
  for (long n = 0; n < T; n++) s->nodeVF[n] *= 0.125;
  int idx = 0;
  for (long n = 0; n < T; n++) s->sdof[n] = -1;
  for (int z = 1; z < s->Z - 1; z++)
    for (int y = 1; y < s->Y - 1; y++)
      for (int x = 1; x < s->X - 1; x++) {
        long index = NIDX(x, y, z);
        s->sdof[index] = (s->solidMass[index] > 0) ? idx++ : -1;
      }
  if (idx != s->nSolid || !s->solidUnitForce) {
    free_solid_vectors(s);
    long S3 = 3L * idx;
    s->solidUnitForce = xcalloc(S3, 8);
    s->solidMv = xcalloc(S3, 8);
    s->damped = xcalloc(S3, 8);
    s->solidV0 = xcalloc(S3, 8);
    s->solidPC = xcalloc(S3, 8);
    s->solidB1 = xcalloc(S3, 8);
    s->sysDiag = xcalloc(S3, 8);
  }
  s->nSolid = idx;
}

/* DEFOR_SOLID_3D::init (DEFOR_SOLID_3D.cpp:269-331) and
 * COUPLED_INTEGRATOR_3D::init (COUPLED_INTEGRATOR_3D.cpp:104-135). */
int esfo_init(esfo_scene* s) {
  if (!s || s->inited || s->ns == 0) return ESF_ERR_STATE;
  if (s->p.mass_sample_dh <= 0 || (int)(s->dh / s->p.mass_sample_dh) < 1) return ESF_ERR_INVALID_ARG;
  for (int i = 0; i < s->ns; i++) {
    solid_t* d = s->s[i];
    d->xmin = d->ymin = d->zmin = 0;
    d->xmax = s->X;
    d->ymax = s->Y;
    d->zmax = s->Z;
    d->tmin[0] = d->tmin[1] = d->tmin[2] = 0;
    d->tmax[0] = s->X;
    d->tmax[1] = s->Y;
    d->tmax[2] = s->Z;
    compute_solid_mass(s, d, 0);
    compute_sdf(s, d);
    init_particles(s, d);
    advect_mesh(s, d);
  }
  gather_solid_masses(s);
  for (int i = 0; i < s->ns; i++) recover_velocity(s, s->s[i], s->vel);
  int idx = 0;
  for (int z = 1; z < s->Z - 1; z++)
    for (int y = 1; y < s->Y - 1; y++)
      for (int x = 1; x < s->X - 1; x++) s->dof[NIDX(x, y, z)] = idx++;
  s->inited = 1;
  return ESF_OK;
}

/* --------------------------------------------------------- dot / norm ---- */
/* VectorXd dot/squaredNorm in Eigen 3.2's SSE2 order: two 2-lane packet
 * accumulators over 4-element strides, then the tail
 * (Eigen/src/Core/Redux.h:193-243). */
static double edot(const double* a, const double* b, long n) {
  if (n <= 0) return 0.0;
  long aS2 = (n / 4) * 4, aS = (n / 2) * 2;
  double res;
  if (aS) {
    double p0a = a[0] * b[0], p0b = a[1] * b[1];
    if (aS > 2) {
      double p1a = a[2] * b[2], p1b = a[3] * b[3];
      for (long i = 4; i < aS2; i += 4) {
        p0a = p0a + a[i] * b[i];
        p0b = p0b + a[i + 1] * b[i + 1];
        p1a = p1a + a[i + 2] * b[i + 2];
        p1b = p1b + a[i + 3] * b[i + 3];
      }
      p0a = p0a + p1a;
      p0b = p0b + p1b;
      if (aS > aS2) {
        p0a = p0a + a[aS2] * b[aS2];
        p0b = p0b + a[aS2 + 1] * b[aS2 + 1];
      }
    }
    res = p0a + p0b;
    for (long i = aS; i < n; i++) res = res + a[i] * b[i];
  } else {
    res = a[0] * b[0];
    for (long i = 1; i < n; i++) res = res + a[i] * b[i];
  }
  return res;
}
static double enorm(const double* a, long n) { return sqrt(edot(a, a, n)); }

/* --------------------------------------------------- pressure operator --- */
/* getMatVecMult (COUPLED_INTEGRATOR_3D.cpp:638-660) with J from
 * computeDivergenceConstraintJacobian (:230-283) applied matrix-free in J's
 * CSR order: mid = J^T in sums each DOF's 8 cells in increasing cell index,
 * out[c] sums the cell's DOF corners in corner order i = 0..7, d = 0..2,
 * each term (sign * mid) * minv. */
static void pressure_apply_d(int X, int Y, int Z, const int* dof, const double* minvD,
                             const double* in, double* out, double* mid) {
  const long slab = (long)X * Y;
  const long cX = X - 1, cS = (long)(X - 1) * (Y - 1);
#pragma omp parallel for schedule(static)
  for (int z = 1; z < Z - 1; z++)
    for (int y = 1; y < Y - 1; y++)
      for (int x = 1; x < X - 1; x++) {
        int k = dof[x + y * X + z * slab];
        double m0 = 0, m1 = 0, m2 = 0;
        /* cells in increasing index: corner i = 7..0 of cell n - offsets[i] */
        for (int i = 7; i >= 0; i--) {
          int cx = x - (i & 1), cy = y - ((i >> 1) & 1), cz = z - ((i >> 2) & 1);
          double l = in[cx + cy * cX + cz * cS];
          double sx = (i % 2 == 0) ? -1 : 1, sy = (i % 4 <= 1) ? -1 : 1, sz = (i < 4) ? -1 : 1;
          m0 += sx * l;
          m1 += sy * l;
          m2 += sz * l;
        }
        mid[3 * k] = m0;
        mid[3 * k + 1] = m1;
        mid[3 * k + 2] = m2;
      }
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Z - 1; z++)
    for (int y = 0; y < Y - 1; y++)
      for (int x = 0; x < X - 1; x++) {
        double acc = 0;
        for (int i = 0; i < 8; i++) {
          int nx = x + (i & 1), ny = y + ((i >> 1) & 1), nz = z + ((i >> 2) & 1);
          int k = dof[nx + ny * X + nz * slab];
          if (k < 0) continue;
          double sx = (i % 2 == 0) ? -1 : 1, sy = (i % 4 <= 1) ? -1 : 1, sz = (i < 4) ? -1 : 1;
          acc += sx * mid[3 * k] * minvD[3 * k];
          acc += sy * mid[3 * k + 1] * minvD[3 * k + 1];
          acc += sz * mid[3 * k + 2] * minvD[3 * k + 2];
        }
        out[x + y * cX + z * cS] = acc;
      }
}

typedef void (*matvec_fn)(void* ctx, const double* in, double* out);

/* CONJUGATE_RESIDUAL::solvePCR, matrix-free variant with warm start
 * (CONJUGATE_RESIDUAL.inl:109-192) and Jacobi preconditioner
 * (JACOBI_PRECONDITIONER.h:35-37). Work arrays w[0..5] of length n. */
static int pcr_solve(matvec_fn A, void* ctx, const double* diag, const double* b, double* x,
                     long n, double eps, int maxIt, int zeroStart, double** w, int* iters,
                     double* relres) {
  double *q = w[0], *r = w[1], *d = w[2], *sv = w[3], *Ap = w[4], *tmp = w[5];
  if (zeroStart) memset(x, 0, n * 8);
  A(ctx, x, q);
  _Pragma("omp parallel for schedule(static)")
  for (long i = 0; i < n; i++) r[i] = b[i] - q[i];
  _Pragma("omp parallel for schedule(static)")
  for (long i = 0; i < n; i++) d[i] = r[i] / diag[i];
  memcpy(r, d, n * 8);
  A(ctx, r, sv);
  memcpy(Ap, sv, n * 8);
  double deltaNew = edot(r, sv, n);
  double bNorm = enorm(b, n);
  int converged = 0, i = 0;
  double tmpNorm = NAN;
  for (; i < maxIt && !converged; i++) {
    _Pragma("omp parallel for schedule(static)")
    for (long k = 0; k < n; k++) q[k] = Ap[k] / diag[k];
    double alpha = edot(Ap, q, n);
    if (fabs(alpha) > 0.0) alpha = deltaNew / alpha;
    _Pragma("omp parallel for schedule(static)")
    for (long k = 0; k < n; k++) x[k] += alpha * d[k];
    _Pragma("omp parallel for schedule(static)")
    for (long k = 0; k < n; k++) r[k] -= alpha * q[k];
    A(ctx, r, sv);
    double deltaOld = deltaNew;
    deltaNew = edot(r, sv, n);
    double beta = deltaNew / deltaOld;
    _Pragma("omp parallel for schedule(static)")
    for (long k = 0; k < n; k++) d[k] *= beta;
    _Pragma("omp parallel for schedule(static)")
    for (long k = 0; k < n; k++) d[k] += r[k];
    _Pragma("omp parallel for schedule(static)")
    for (long k = 0; k < n; k++) Ap[k] *= beta;
    _Pragma("omp parallel for schedule(static)")
    for (long k = 0; k < n; k++) Ap[k] += sv[k];
    if (i > 0 && i % 5 == 0) {
      A(ctx, x, tmp);
      _Pragma("omp parallel for schedule(static)")
      for (long k = 0; k < n; k++) tmp[k] -= b[k];
      tmpNorm = enorm(tmp, n);
      if (tmpNorm < eps * bNorm) {
        converged = 1;
        break;
      }
    }
  }
  if (iters) *iters = i;
  if (relres) {
    if (!(tmpNorm == tmpNorm)) {
      A(ctx, x, tmp);
      _Pragma("omp parallel for schedule(static)")
      for (long k = 0; k < n; k++) tmp[k] -= b[k];
      tmpNorm = enorm(tmp, n);
    }
    *relres = bNorm > 0 ? tmpNorm / bNorm : tmpNorm;
  }
  return converged;
}

typedef struct {
  int X, Y, Z;
  const int* dof;
  const double* minvD;
  double* mid;
} pctx;
static void pressure_mv(void* c, const double* in, double* out) {
  pctx* p = (pctx*)c;
  pressure_apply_d(p->X, p->Y, p->Z, p->dof, p->minvD, in, out, p->mid);
}

typedef struct {
  const int* Ap;
  const int* Aj;
  const double* Ax;
  long n;
} sctx;
/* CONJUGATE_RESIDUAL::parallelMatVecMult (CONJUGATE_RESIDUAL.inl:31-44). */
static void csr_mv(void* c, const double* in, double* out) {
  sctx* p = (sctx*)c;
  for (long k = 0; k < p->n; k++) {
    double acc = 0;
    for (int e = p->Ap[k]; e < p->Ap[k + 1]; e++) acc += p->Ax[e] * in[p->Aj[e]];
    out[k] = acc;
  }
}

static int* interior_dof_map(const esf_grid* g) {
  int X = g->xRes, Y = g->yRes, Z = g->zRes;
  int* dof = (int*)xcalloc((size_t)X * Y * Z, 4);
  long slab = (long)X * Y;
  for (long i = 0; i < slab * Z; i++) dof[i] = -1;
  int idx = 0;
  for (int z = 1; z < Z - 1; z++)
    for (int y = 1; y < Y - 1; y++)
      for (int x = 1; x < X - 1; x++) dof[x + y * X + z * slab] = idx++;
  return dof;
}
static double* node_to_dof_minv(const esf_grid* g, const int* dof, const double* mnode) {
  long T = (long)g->xRes * g->yRes * g->zRes;
  long D = 3L * (g->xRes - 2) * (g->yRes - 2) * (g->zRes - 2);
  double* m = (double*)xcalloc(D, 8);
  for (long n = 0; n < T; n++)
    if (dof[n] >= 0)
      for (int k = 0; k < 3; k++) m[3 * dof[n] + k] = mnode[n];
  return m;
}

int esfo_pressure_apply(const esf_grid* g, const double* mnode, const double* in, double* out) {
  if (!g || !mnode || !in || !out) return ESF_ERR_INVALID_ARG;
  int* dof = interior_dof_map(g);
  double* minv = node_to_dof_minv(g, dof, mnode);
  long D = 3L * (g->xRes - 2) * (g->yRes - 2) * (g->zRes - 2);
  double* mid = (double*)xcalloc(D, 8);
  pressure_apply_d(g->xRes, g->yRes, g->zRes, dof, minv, in, out, mid);
  free(dof);
  free(minv);
  free(mid);
  return ESF_OK;
}

int esfo_pressure_solve(const esf_grid* g, const double* mnode, const double* diag,
                        const double* b, double* x, double eps, int maxIt, int* iters,
                        double* relres) {
  if (!g || !mnode || !diag || !b || !x) return ESF_ERR_INVALID_ARG;
  int* dof = interior_dof_map(g);
  double* minv = node_to_dof_minv(g, dof, mnode);
  long D = 3L * (g->xRes - 2) * (g->yRes - 2) * (g->zRes - 2);
  long R = (long)(g->xRes - 1) * (g->yRes - 1) * (g->zRes - 1);
  double* mid = (double*)xcalloc(D, 8);
  double* w[6];
  for (int i = 0; i < 6; i++) w[i] = (double*)xcalloc(R, 8);
  pctx c = {g->xRes, g->yRes, g->zRes, dof, minv, mid};
  int conv = pcr_solve(pressure_mv, &c, diag, b, x, R, eps, maxIt, 0, w, iters, relres);
  for (int i = 0; i < 6; i++) free(w[i]);
  free(dof);
  free(minv);
  free(mid);
  return conv ? ESF_OK : ESF_ERR_NUMERIC;
}

/* ------------------------------------------------------ the step ---------- */
typedef struct {
  int row, col;
  long seq;
  double v;
} trip;
static int trip_cmp(const void* a, const void* b) {
  const trip* x = (const trip*)a;
  const trip* y = (const trip*)b;
  if (x->row != y->row) return x->row < y->row ? -1 : 1;
  if (x->col != y->col) return x->col < y->col ? -1 : 1;
  return (x->seq < y->seq) ? -1 : (x->seq > y->seq);
}
typedef struct {
  trip* t;
  long n, cap;
} tripvec;
static void tpush(tripvec* v, int r, int c, double x) {
  if (v->n == v->cap) {
    v->cap = v->cap ? 2 * v->cap : 4096;
    v->t = (trip*)realloc(v->t, v->cap * sizeof(trip));
    if (!v->t) abort();
  }
  v->t[v->n].row = r;
  v->t[v->n].col = c;
  v->t[v->n].seq = v->n;
  v->t[v->n].v = x;
  v->n++;
}

/* ||A|| of a 3x3 matrix (Eigen's norm()): the squares in column-major order
 * summed as two-lane packets ((a0,a1)+(a2,a3)) + ((a4,a5)+(a6,a7)), the lanes
 * added, then the ninth square. */
static double m3_norm(const m3* a) {
  double q[9];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) q[j * 3 + i] = a->m[i][j] * a->m[i][j];
  double l0 = (q[0] + q[2]) + (q[4] + q[6]);
  double l1 = (q[1] + q[3]) + (q[5] + q[7]);
  return sqrt((l0 + l1) + q[8]);
}
/* MATRIX3_FIELD_3D::interpolate_value (MATRIX3_FIELD_3D.h:127-135): the
 * material cell holding a rest position, clamped to the grid. */
static long fp_index(const solid_t* d, const double p[3]) {
  int c[3];
  for (int k = 0; k < 3; k++) {
    double x = (p[k] - d->porig[k]) / d->pdh;
    int i = (int)floor(x);
    if (i <= 0) i = 0;
    else if (i >= d->pres[k] - 1) i = d->pres[k] - 1;
    c[k] = i;
  }
  return ((long)c[2] * d->pres[1] + c[1]) * d->pres[0] + c[0];
}
static m3 fp_get(const double* f, long c) {
  m3 r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) r.m[i][j] = f[c * 9 + i * 3 + j];
  return r;
}

/* computeStiffnessMatrixAndMaterialForce (DEFOR_SOLID_3D.cpp:697-871) for
 * an elastic solid, and computePFPxhat (:684-695) folded in. */
static double stiffness(esfo_scene* s, solid_t* d, double* force, tripvec* tl, const int* map) {
  const long off[8] = {0, 1, s->X, s->X + 1, s->slab, s->slab + 1, s->slab + s->X,
                       s->slab + s->X + 1};
  const long pn = d->plastic ? (long)d->pres[0] * d->pres[1] * d->pres[2] : 0;
  if (pn) memset(d->fpSet, 0, pn);
  const double dh = s->dh;
  double energy = 0;
  corot mat;
  mat.lambda = d->lambda;
  mat.mu = d->mu;
  static double K[24][24];
  for (int z = d->tmin[2]; z < d->tmax[2] - 1; z++)
    for (int y = d->tmin[1]; y < d->tmax[1] - 1; y++)
      for (int x = d->tmin[0]; x < d->tmax[0] - 1; x++) {
        if (d->valid[VIDX(x, y, z)] != 1) continue;
        long index = NIDX(x, y, z);
        double c[8][3];
        gather_corners(s, d->u, index, c);
        m3 F;
        double Jinv = 1.0 / compute_F(d, c, &F);
        corot_init(&mat, &F);
        m3 P = corot_pk1(&mat);
        m3 JP;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) JP.m[i][j] = Jinv * P.m[i][j];
        m3 cs = m3_mul_bt(&JP, &F);
        /* plasticity (DEFOR_SOLID_3D.cpp:765-791): above the yield stress the
         * elastic part F FpInv is used, and FpInv is updated by a flow step
         * on the singular values; the updates are written after the sweep,
         * the last cell in sweep order winning for a material cell */
        if (d->plastic && m3_norm(&cs) > d->yield) {
          double rp[3] = {0, 0, 0};
          for (int i = 0; i < 8; i++)
            for (int k = 0; k < 3; k++) rp[k] += d->X[3 * (index + off[i]) + k];
          for (int k = 0; k < 3; k++) rp[k] /= 8;
          const long mc = fp_index(d, rp);
          m3 Fp = fp_get(d->FpInv, mc);
          F = m3_mul(&F, &Fp);
          corot_init(&mat, &F);
          P = corot_pk1(&mat);
          for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) JP.m[i][j] = Jinv * P.m[i][j];
          cs = m3_mul_bt(&JP, &F);
          const double cNorm = m3_norm(&cs);
          if (cNorm > d->yield) {
            const double gamma = s->p.flow_rate * (cNorm - d->yield) / cNorm;
            const double cr = cbrt(1.0 / fmax(fabs(Jinv), 1e-3));
            m3 Fh = mat.Fhat;
            for (int i = 0; i < 3; i++) Fh.m[i][i] = pow(Fh.m[i][i] / cr, -gamma);
            m3 VF = m3_mul(&mat.V, &Fh);
            m3 dFp = m3_mul_bt(&VF, &mat.V);
            m3 nFp = m3_mul(&dFp, &Fp);
            int bad = 0;
            for (int i = 0; i < 3; i++)
              for (int j = 0; j < 3; j++) bad |= nFp.m[i][j] != nFp.m[i][j];
            if (!bad) {
              for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) d->FpNew[mc * 9 + i * 3 + j] = nFp.m[i][j];
              d->fpSet[mc] = 1;
            }
          }
        }
        double GF[8][3]; /* _G * F */
        for (int i = 0; i < 8; i++)
          for (int j = 0; j < 3; j++)
            GF[i][j] = (d->G[i][0] * F.m[0][j] + d->G[i][1] * F.m[1][j]) + d->G[i][2] * F.m[2][j];
        double nf[3][8]; /* -= cauchy * G^T * dh * dh * dh */
        for (int r = 0; r < 3; r++)
          for (int m = 0; m < 8; m++) {
            double t = (cs.m[r][0] * d->G[m][0] + cs.m[r][1] * d->G[m][1]) + cs.m[r][2] * d->G[m][2];
            nf[r][m] = 0.0 - ((t * dh) * dh) * dh;
          }
        energy += corot_energy(&mat) * dh * dh * dh;
        memset(K, 0, sizeof K);
        for (int k = 0; k < 24; k++) {
          long col = index + off[k / 3];
          if (d->mass[col] == 0) continue;
          int ci = k / 3, cj = k % 3;
          m3 dF;
          memset(&dF, 0, sizeof dF);
          for (int cc = 0; cc < 3; cc++) dF.m[cj][cc] = GF[ci][cc];
          m3 dP = corot_dpk(&mat, &dF);
          for (int m = 0; m < 8; m++)
            for (int r = 0; r < 3; r++) {
              double t = (dP.m[r][0] * GF[m][0] + dP.m[r][1] * GF[m][1]) + dP.m[r][2] * GF[m][2];
              K[m * 3 + r][k] += (((t * Jinv) * dh) * dh) * dh;
            }
        }
        for (int i = 0; i < 8; i++) {
          int idx = map[index + off[i]];
          if (idx >= 0)
            for (int r = 0; r < 3; r++) force[3 * idx + r] += nf[r][i];
        }
        for (int i = 0; i < 24; i++) {
          long col = index + off[i / 3];
          if (d->mass[col] == 0) continue;
          if (map[col] < 0) continue;
          int newCol = map[col] * 3 + i % 3;
          for (int k = 0; k < 24; k++) {
            long row = index + off[k / 3];
            if (d->mass[row] == 0) continue;
            if (map[row] < 0) continue;
            tpush(tl, map[row] * 3 + k % 3, newCol, K[k][i]);
          }
        }
      }
  for (long c = 0; c < pn; c++)
    if (d->fpSet[c]) memcpy(d->FpInv + c * 9, d->FpNew + c * 9, 72);
  return energy;
}

/* DEFOR_SOLID_3D::computeMV (DEFOR_SOLID_3D.cpp:873-889). */
static double compute_mv(esfo_scene* s, solid_t* d, double* mv, const int* map) {
  double energy = 0;
  for (int z = d->zmin; z < d->zmax - 1; z++)
    for (int y = d->ymin; y < d->ymax - 1; y++)
      for (int x = d->xmin; x < d->xmax - 1; x++) {
        long n = NIDX(x, y, z);
        int idx = map[n];
        if (idx >= 0) {
          const double* v = d->vel + 3 * n;
          for (int k = 0; k < 3; k++) mv[3 * idx + k] += d->mass[n] * v[k];
          energy += 0.5 * d->mass[n] * (v[0] * v[0] + (v[1] * v[1] + v[2] * v[2]));
        }
      }
  return energy;
}

/* DEFOR_SOLID_3D::gridToParticle (DEFOR_SOLID_3D.cpp:891-1034). */
static void bspline(double dd, double* n) {
  double a = fabs(dd);
  double c = fabs(pow(dd, 3));
  if (a < 1) *n = 0.5 * c - dd * dd + 2.0 / 3;
  else if (a < 2) *n = -1.0 / 6 * c + dd * dd - 2 * a + 4.0 / 3;
  else *n = 0;
}
static void grid_to_particle(esfo_scene* s, solid_t* d) {
  const double alpha = s->p.flip_alpha;
  const double wallN[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
  const double bnd[6] = {s->o[0], s->o[1], s->o[2], s->o[0] + s->dh * (s->X - 1),
                         s->o[1] + s->dh * (s->Y - 1), s->o[2] + s->dh * (s->Z - 1)};
  for (long c = 0; c < d->np; c++) {
    double* P = d->part + 10 * c;
    double fx = (P[0] - s->o[0]) / s->dh, fy = (P[1] - s->o[1]) / s->dh, fz = (P[2] - s->o[2]) / s->dh;
    int i = (int)floor(fx) - 1, j = (int)floor(fy) - 1, k = (int)floor(fz) - 1;
    double pic[3] = {0, 0, 0}, flip[3] = {0, 0, 0};
    for (int r = k; r < k + 4; r++)
      for (int t = j; t < j + 4; t++)
        for (int sx = i; sx < i + 4; sx++) {
          if (sx < 0 || t < 0 || r < 0 || sx > s->X - 1 || t > s->Y - 1 || r > s->Z - 1) continue;
          long n = NIDX(sx, t, r);
          if (d->mass[n] == 0) continue;
          double diff[3], nn[3];
          for (int q = 0; q < 3; q++) diff[q] = s->dhInv * (P[q] - s->o[q]);
          diff[0] -= sx;
          diff[1] -= t;
          diff[2] -= r;
          for (int q = 0; q < 3; q++) bspline(diff[q], &nn[q]);
          double w = nn[0] * nn[1] * nn[2];
          for (int q = 0; q < 3; q++) {
            pic[q] += d->vel[3 * n + q] * w;
            flip[q] += (d->vel[3 * n + q] - d->vws[3 * n + q]) * w;
          }
        }
    for (int q = 0; q < 3; q++) {
      flip[q] += P[3 + q];
      P[3 + q] = (1 - alpha) * pic[q] + alpha * flip[q];
    }
  }
  const double thickness = s->p.contact_safe_distance;
  const double wallThickness = s->p.wall_thickness;
  const double spring = s->p.contact_spring_stiffness;
  const double friction = s->p.friction;
  (void)thickness;
  for (long c = 0; c < d->np; c++) {
    double* P = d->part + 10 * c;
    double fx = (P[0] - s->o[0]) / s->dh, fy = (P[1] - s->o[1]) / s->dh, fz = (P[2] - s->o[2]) / s->dh;
    int i = (int)floor(fx), j = (int)floor(fy), k = (int)floor(fz);
    i = imin(imax(i, 0), s->X - 2);
    j = imin(imax(j, 0), s->Y - 2);
    k = imin(imax(k, 0), s->Z - 2);
    for (int y = 0; y < s->ns; y++) {
      solid_t* nb = s->s[y];
      if (nb == d) continue;
      if (I1(s, nb->phi, P) > 2) continue;
      s->status = ESF_ERR_UNSUPPORTED; /* solid-solid contact not restated */
    }
    for (int b = 0; b < 6; b++) {
      double dist = fabs(P[b % 3] - bnd[b]);
      if (dist < wallThickness) {
        double overlap = wallThickness - dist;
        int xi = i, yi = j, zi = k;
        if (b == 0) xi = 0;
        else if (b == 3) xi = s->X - 1;
        if (b == 1) yi = 0;
        else if (b == 4) yi = s->Y - 1;
        if (b == 2) zi = 0;
        else if (b == 5) zi = s->Z - 1;
        const double* vo = d->vel + 3 * NIDX(xi, yi, zi);
        double vrel[3] = {P[3] - vo[0], P[4] - vo[1], P[5] - vo[2]};
        double vn = (vrel[0] * wallN[b][0] + vrel[1] * wallN[b][1]) + vrel[2] * wallN[b][2];
        if (vn <= 0) {
          double impulse = -dmin(d->dt * spring * overlap, P[9] * (0.1 * overlap / d->dt - vn));
          double dvn = -impulse / P[9];
          double vt[3];
          for (int q = 0; q < 3; q++) vt[q] = vrel[q] - vn * wallN[b][q];
          double vtn = sqrt(vt[0] * vt[0] + (vt[1] * vt[1] + vt[2] * vt[2]));
          double sc = dmax(0.1 - friction * dvn / vtn, 0.0);
          for (int q = 0; q < 3; q++) P[3 + q] = ((vn + dvn) * wallN[b][q] + sc * vt[q]) + vo[q];
          break;
        }
      }
    }
    for (int q = 0; q < 3; q++) P[q] += P[3 + q] * d->dt;
  }
}

/* DEFOR_SOLID_3D::particleToGrid (DEFOR_SOLID_3D.cpp:1036-1107), serial
 * accumulation in particle order. */
static void particle_to_grid(esfo_scene* s, solid_t* d) {
  long T = s->total;
  double* acc = (double*)xcalloc(T * 4, 8);
  unsigned char* touched = (unsigned char*)xcalloc(T, 1);
  for (long c = 0; c < d->np; c++) {
    const double* P = d->part + 10 * c;
    double fx = (P[0] - s->o[0]) / s->dh, fy = (P[1] - s->o[1]) / s->dh, fz = (P[2] - s->o[2]) / s->dh;
    int i = (int)floor(fx) - 1, j = (int)floor(fy) - 1, k = (int)floor(fz) - 1;
    for (int r = k; r < k + 4; r++)
      for (int t = j; t < j + 4; t++)
        for (int sx = i; sx < i + 4; sx++) {
          if (sx < 0 || t < 0 || r < 0 || sx > s->X - 1 || t > s->Y - 1 || r > s->Z - 1) continue;
          double diff[3], nn[3];
          for (int q = 0; q < 3; q++) diff[q] = s->dhInv * (P[q] - s->o[q]);
          diff[0] -= sx;
          diff[1] -= t;
          diff[2] -= r;
          for (int q = 0; q < 3; q++) bspline(diff[q], &nn[q]);
          double w = nn[0] * nn[1] * nn[2];
          long n = NIDX(sx, t, r);
          if (!touched[n]) {
            touched[n] = 1;
            for (int q = 0; q < 3; q++) acc[4 * n + q] = w * P[3 + q];
            acc[4 * n + 3] = w;
          } else {
            for (int q = 0; q < 3; q++) acc[4 * n + q] += w * P[3 + q];
            acc[4 * n + 3] += w;
          }
        }
  }
  memset(d->mass, 0, T * 8);
  for (long n = 0; n < T; n++) {
    if (!touched[n] || acc[4 * n + 3] < s->p.flip_cutoff) continue;
    for (int q = 0; q < 3; q++) d->vel[3 * n + q] = acc[4 * n + q] / acc[4 * n + 3];
    d->mass[n] = 1;
  }
  free(acc);
  free(touched);
}

/* DEFOR_SOLID_3D::sweepOnePass (DEFOR_SOLID_3D.cpp:457-519), including its
 * pass-long solvableX/Y/Z flags. */
static void sweep_one_pass(esfo_scene* s, solid_t* d, double* f, int i0, int i1, int j0, int j1,
                           int k0, int k1) {
  int di = (i0 < i1) ? 1 : -1, dj = (j0 < j1) ? 1 : -1, dk = (k0 < k1) ? 1 : -1;
  int sX = 1, sY = 1, sZ = 1;
  const double* ph = d->phi;
  for (int k = k0; k != k1; k += dk)
    for (int j = j0; j != j1; j += dj)
      for (int i = i0; i != i1; i += di) {
        long n = NIDX(i, j, k);
        if (d->mass[n] != 0) continue;
        double dp = ph[n] - ph[NIDX(i - di, j, k)];
        double dpn = ph[n] - ph[NIDX(i + di, j, k)];
        if (dp < 0) {
          if (dpn >= 0) continue;
          sX = 0;
        }
        double dq = ph[n] - ph[NIDX(i, j - dj, k)];
        double dqn = ph[n] - ph[NIDX(i, j + dj, k)];
        if (dq < 0) {
          if (dqn >= 0) continue;
          sY = 0;
        }
        double dr = ph[n] - ph[NIDX(i, j, k - dk)];
        double drn = ph[n] - ph[NIDX(i, j, k + dk)];
        if (dr < 0) {
          if (drn >= 0) continue;
          sZ = 0;
        }
        if (!sX) dp = 0;
        if (!sY) dq = 0;
        if (!sZ) dr = 0;
        double alpha, beta;
        if (dp + dq + dr < 1e-3) {
          alpha = 0.333;
          beta = 0.333;
        } else {
          alpha = dp / (dp + dq + dr);
          beta = dq / (dp + dq + dr);
        }
        long a = NIDX(i - di, j, k), b = NIDX(i, j - dj, k), c = NIDX(i, j, k - dk);
        for (int q = 0; q < 3; q++)
          f[3 * n + q] = (alpha * f[3 * a + q] + beta * f[3 * b + q]) + (1 - alpha - beta) * f[3 * c + q];
      }
}

/* sweepVectorField (DEFOR_SOLID_3D.cpp:521-564). */
static void sweep_vector_field(esfo_scene* s, solid_t* d, double* f) {
  int xn = d->xmin, xm = d->xmax, yn = d->ymin, ym = d->ymax, zn = d->zmin, zm = d->zmax;
  sweep_one_pass(s, d, f, xn + 1, xm - 1, yn + 1, ym - 1, zn + 1, zm - 1);
  sweep_one_pass(s, d, f, xn + 1, xm - 1, ym - 2, yn, zn + 1, zm - 1);
  sweep_one_pass(s, d, f, xm - 2, xn, yn + 1, ym - 1, zn + 1, zm - 1);
  sweep_one_pass(s, d, f, xm - 2, xn, ym - 2, yn, zn + 1, zm - 1);
  sweep_one_pass(s, d, f, xn + 1, xm - 1, yn + 1, ym - 1, zm - 2, zn);
  sweep_one_pass(s, d, f, xn + 1, xm - 1, ym - 2, yn, zm - 2, zn);
  sweep_one_pass(s, d, f, xm - 2, xn, yn + 1, ym - 1, zm - 2, zn);
  sweep_one_pass(s, d, f, xm - 2, xn, ym - 2, yn, zm - 2, zn);
  const double* m = d->mass;
#define CP(dst, src) \
  for (int q = 0; q < 3; q++) f[3 * (dst) + q] = f[3 * (src) + q]
  for (int i = xn; i < xm; i++)
    for (int j = yn; j < ym; j++) {
      if (m[NIDX(i, j, zn)] == 0) CP(NIDX(i, j, zn), NIDX(i, j, zn + 1));
      if (m[NIDX(i, j, zm - 1)] == 0) CP(NIDX(i, j, zm - 1), NIDX(i, j, zm - 2));
    }
  for (int i = xn; i < xm; i++)
    for (int k = zn; k < zm; k++) {
      if (m[NIDX(i, yn, k)] == 0) CP(NIDX(i, yn, k), NIDX(i, yn + 1, k));
      if (m[NIDX(i, ym - 1, k)] == 0) CP(NIDX(i, ym - 1, k), NIDX(i, ym - 2, k));
    }
  for (int j = yn; j < ym; j++)
    for (int k = zn; k < zm; k++) {
      if (m[NIDX(xn, j, k)] == 0) CP(NIDX(xn, j, k), NIDX(xn + 1, j, k));
      if (m[NIDX(xm - 1, j, k)] == 0) CP(NIDX(xm - 1, j, k), NIDX(xm - 2, j, k));
    }
#undef CP
}

/* DEFOR_SOLID_3D::finalizeSolution() (DEFOR_SOLID_3D.cpp:1198-1233) with
 * advectField (:1108-1123). */
static void solid_finalize(esfo_scene* s, solid_t* d) {
  long T = s->total;
  for (long i = 0; i < T; i++)
    for (int q = 0; q < 3; q++) d->u[3 * i + q] += d->vel[3 * i + q] * d->dt;
  for (int z = 0; z < s->Z; z++)
    for (int y = 0; y < s->Y; y++)
      for (int x = 0; x < s->X; x++) {
        long n = NIDX(x, y, z);
        double node[3] = {(double)x, (double)y, (double)z};
        for (int q = 0; q < 3; q++) node[q] = node[q] * s->dh + s->o[q];
        double np[3];
        for (int q = 0; q < 3; q++) np[q] = node[q] - d->vel[3 * n + q] * d->dt;
        I3(s, d->u, np, d->tmp3 + 3 * n);
      }
  double* t = d->u;
  d->u = d->tmp3;
  d->tmp3 = t;
  double* u = d->u;
#define EX(a, b, c) \
  for (int q = 0; q < 3; q++) u[3 * (a) + q] = 2 * u[3 * (b) + q] - u[3 * (c) + q]
  for (int x = d->xmin; x < d->xmax; x++)
    for (int y = d->ymin; y < d->ymax; y++) {
      EX(NIDX(x, y, d->zmin), NIDX(x, y, d->zmin + 1), NIDX(x, y, d->zmin + 2));
      EX(NIDX(x, y, d->zmax - 1), NIDX(x, y, d->zmax - 2), NIDX(x, y, d->zmax - 3));
    }
  for (int x = d->xmin; x < d->xmax; x++)
    for (int z = d->zmin; z < d->zmax; z++) {
      EX(NIDX(x, d->ymin, z), NIDX(x, d->ymin + 1, z), NIDX(x, d->ymin + 2, z));
      EX(NIDX(x, d->ymax - 1, z), NIDX(x, d->ymax - 2, z), NIDX(x, d->ymax - 3, z));
    }
  for (int y = d->ymin; y < d->ymax; y++)
    for (int z = d->zmin; z < d->zmax; z++) {
      EX(NIDX(d->xmin, y, z), NIDX(d->xmin + 1, y, z), NIDX(d->xmin + 2, y, z));
      EX(NIDX(d->xmax - 1, y, z), NIDX(d->xmax - 2, y, z), NIDX(d->xmax - 3, y, z));
    }
#undef EX
  for (int z = 0; z < s->Z; z++)
    for (int y = 0; y < s->Y; y++)
      for (int x = 0; x < s->X; x++) {
        long n = NIDX(x, y, z);
        double pos[3] = {x * s->dh, y * s->dh, z * s->dh};
        for (int q = 0; q < 3; q++) d->X[3 * n + q] = pos[q] + (s->o[q] - u[3 * n + q]);
      }
  memcpy(d->vws, d->vel, T * 24);
}

/* COUPLED_INTEGRATOR_3D::CFL (COUPLED_INTEGRATOR_3D.cpp:88-102). */
static double cfl(esfo_scene* s, double alpha) {
  double dt = 1e9;
  for (int z = 1; z < s->Z - 1; z++)
    for (int y = 1; y < s->Y - 1; y++)
      for (int x = 1; x < s->X - 1; x++) {
        long n = NIDX(x, y, z);
        if (s->solidMass[n] > 0) {
          const double* v = s->vel + 3 * n;
          double vmax = dmax(dmax(fabs(v[0]), fabs(v[1])), fabs(v[2])) * s->dhInv;
          dt = dmin(dt, alpha / vmax);
        }
      }
  return dmin(dt, s->defaultDt);
}

static void vertex_aabb(const solid_t* d, double* mn, double* mx) {
  for (int k = 0; k < 3; k++) {
    mn[k] = DBL_MAX;
    mx[k] = -DBL_MAX;
  }
  for (int t = 0; t < d->ntri * 3; t++) {
    const double* v = d->verts + 3 * d->tris[t];
    for (int k = 0; k < 3; k++) {
      if (v[k] < mn[k]) mn[k] = v[k];
      if (v[k] > mx[k]) mx[k] = v[k];
    }
  }
}
/* aabb::inside (src/deformCD/aabb.cpp:135-143) */
static int box_inside(const double* bmn, const double* bmx, const double* p) {
  for (int k = 0; k < 3; k++)
    if (p[k] < bmn[k] || p[k] > bmx[k]) return 0;
  return 1;
}
static int solids_overlap(const solid_t* a, const solid_t* b) {
  for (int ta = 0; ta < a->ntri; ta++) {
    double amn[3], amx[3];
    for (int k = 0; k < 3; k++) {
      amn[k] = DBL_MAX;
      amx[k] = -DBL_MAX;
    }
    for (int v = 0; v < 3; v++)
      for (int k = 0; k < 3; k++) {
        double x = a->verts[3 * a->tris[3 * ta + v] + k];
        amn[k] = dmin(amn[k], x);
        amx[k] = dmax(amx[k], x);
      }
    for (int tb = 0; tb < b->ntri; tb++) {
      int ov = 1;
      for (int k = 0; k < 3 && ov; k++) {
        double bmn = DBL_MAX, bmx = -DBL_MAX;
        for (int v = 0; v < 3; v++) {
          double x = b->verts[3 * b->tris[3 * tb + v] + k];
          bmn = dmin(bmn, x);
          bmx = dmax(bmx, x);
        }
        if (amn[k] > bmx || amx[k] < bmn) ov = 0;
      }
      if (ov) return 1;
    }
  }
  return 0;
}

static void fluid_advect(esfo_scene* s) {
  /* advectFluidVelocityField (COUPLED_INTEGRATOR_3D.cpp:797-826) */
  const double dt = s->dt;
  for (int z = 1; z < s->Z - 1; z++)
    for (int y = 1; y < s->Y - 1; y++)
      for (int x = 1; x < s->X - 1; x++) {
        long n = NIDX(x, y, z);
        if (s->solidMass[n] > 0) continue;
        double node[3] = {x * s->dh + s->o[0], y * s->dh + s->o[1], z * s->dh + s->o[2]};
        double p[3], v[3], np[3];
        for (int q = 0; q < 3; q++) p[q] = node[q] - 0.5 * s->vel[3 * n + q] * dt;
        I3(s, s->vel, p, v);
        for (int q = 0; q < 3; q++) np[q] = node[q] - v[q] * dt;
        double mass = I1(s, s->solidMass, np);
        double newdt = dt / 2;
        while (mass > 0 && newdt > dt / 16) {
          for (int q = 0; q < 3; q++) np[q] += v[q] * newdt;
          newdt /= 2;
          mass = I1(s, s->solidMass, np);
        }
        I3(s, s->vel, np, s->vws + 3 * n);
      }
  double* t = s->vel;
  s->vel = s->vws;
  s->vws = t;
  /* advectField(intensity) (:766-796) */
  memset(s->ws, 0, s->total * 8);
  for (int z = 0; z < s->Z; z++)
    for (int y = 0; y < s->Y; y++)
      for (int x = 0; x < s->X; x++) {
        long n = NIDX(x, y, z);
        if (s->solidMass[n] > 0) continue;
        double node[3] = {x * s->dh + s->o[0], y * s->dh + s->o[1], z * s->dh + s->o[2]};
        const double* v = s->vel + 3 * n;
        double np[3];
        for (int q = 0; q < 3; q++) np[q] = node[q] - v[q] * dt;
        double mass = I1(s, s->solidMass, np);
        double newdt = s->dt / 2;
        while (mass > 0 && newdt > dt / 16) {
          for (int q = 0; q < 3; q++) np[q] += v[q] * newdt;
          newdt /= 2;
          mass = I1(s, s->solidMass, np);
        }
        s->ws[n] = I1(s, s->intensity, np);
      }
  t = s->intensity;
  s->intensity = s->ws;
  s->ws = t;
}

/* COUPLED_INTEGRATOR_3D::stepImplicit (COUPLED_INTEGRATOR_3D.cpp:377-636). */
int esfo_step(esfo_scene* s, esf_step_report* rep) {
  if (!s || !s->inited) return ESF_ERR_STATE;
  s->status = ESF_OK;
  const int X = s->X, Y = s->Y, Z = s->Z;
  const long slab = s->slab;
  const double dh = s->dh;
  /* broad phase (:378-411) */
  int prone = 0;
  for (int i = 0; i < s->ns && !prone; i++) {
    double mn[3], mx[3];
    vertex_aabb(s->s[i], mn, mx);
    if (!(box_inside(s->s[i]->safeMin, s->s[i]->safeMax, mn) &&
          box_inside(s->s[i]->safeMin, s->s[i]->safeMax, mx)))
      prone = 1;
  }
  if (!prone)
    for (int i = 0; i < s->ns - 1 && !prone; i++)
      for (int j = i + 1; j < s->ns && !prone; j++)
        if (solids_overlap(s->s[i], s->s[j])) prone = 1;
  s->dt = cfl(s, prone ? 0.6 : 1.8);
  const double dt = s->dt;

  long D = 3L * s->nInterior, S3 = 3L * s->nSolid, R = s->cells;
  memset(s->unitForce, 0, D * 8);
  memset(s->solidUnitForce, 0, S3 * 8);
  memset(s->solidMv, 0, S3 * 8);
  memset(s->damped, 0, S3 * 8);
  tripvec tl = {0, 0, 0};
  double energy = 0;
  for (int i = 0; i < s->ns; i++) {
    energy += stiffness(s, s->s[i], s->solidUnitForce, &tl, s->sdof);
    energy += compute_mv(s, s->s[i], s->solidMv, s->sdof);
  }
  const double gridSize = 0.5 / dh;
  memset(s->ws, 0, s->total * 8);
  const double rayA = s->p.rayleigh_alpha, rayB = s->p.rayleigh_beta;
  const double damp = 1 + dt * rayA;
  const double* VF = s->nodeVF;
  const double* v = s->vel;
  /* vorticity (:451-497) */
  if (s->vortEps > 0) {
    for (int z = 1; z < Z - 1; z++)
      for (int y = 1; y < Y - 1; y++)
        for (int x = 1; x < X - 1; x++) {
          long n = NIDX(x, y, z);
          if (VF[n] >= 1) continue;
          long up = (VF[n + X] >= 1 || y == Y - 2) ? n : n + X;
          long down = (VF[n - X] >= 1 || y == 1) ? n : n - X;
          double ddy = (up == n || down == n) ? s->dhInv : gridSize;
          long out = (VF[n + slab] >= 1 || z == Z - 2) ? n : n + slab;
          long in = (VF[n - slab] >= 1 || z == 1) ? n : n - slab;
          double ddz = (out == n || in == n) ? s->dhInv : gridSize;
          long right = (VF[n + 1] >= 1 || x == X - 2) ? n : n + 1;
          long left = (VF[n - 1] >= 1 || x == 1) ? n : n - 1;
          double ddx = (right == n || left == n) ? s->dhInv : gridSize;
          double* w = s->vort + 3 * n;
          w[0] = ((v[3 * up + 2] - v[3 * down + 2]) + (-v[3 * out + 1] + v[3 * in + 1])) * ddz;
          w[1] = ((v[3 * out + 0] - v[3 * in + 0]) + (-v[3 * right + 2] + v[3 * left + 2])) * ddx;
          w[2] = ((v[3 * right + 1] - v[3 * left + 1]) + (-v[3 * up + 0] + v[3 * down + 0])) * ddy;
          s->ws[n] = sqrt(w[0] * w[0] + (w[1] * w[1] + w[2] * w[2]));
        }
  }
  /* body forces (:503-606) */
  const double g = s->p.gravity, bu = s->p.buoyancy;
  for (int z = 1; z < Z - 1; z++)
    for (int y = 1; y < Y - 1; y++)
      for (int x = 1; x < X - 1; x++) {
        long n = NIDX(x, y, z);
        int idx = s->dof[n], sidx = s->sdof[n];
        double fm = dmax(1.0 - VF[n], 0.0) * s->fluidDensity * dh * dh * dh;
        double mass = fm + s->solidMass[n];
        double h = dh * y + s->o[1];
        energy += mass * g * h;
        const double* vn = v + 3 * n;
        if (sidx < 0) {
          double mg = mass * g;
          s->unitForce[3 * idx + 0] += mg * 0.0;
          s->unitForce[3 * idx + 1] += mg * -1.0;
          s->unitForce[3 * idx + 2] += mg * 0.0;
          s->unitForce[3 * idx + 1] += bu * fm * s->intensity[n];
          for (int q = 0; q < 3; q++) s->mv[3 * idx + q] = fm * vn[q];
          if (s->vortEps > 0) {
            if (VF[n + X] == 0 && VF[n - X] == 0 && VF[n + 1] == 0 && VF[n - 1] == 0 &&
                VF[n + slab] == 0 && VF[n - slab] == 0) {
              long up = (y == Y - 2) ? n : n + X;
              long down = (VF[n - X] >= 1 || y == 1) ? n : n - X;
              double ddy = (up == n || down == n) ? s->dhInv : gridSize;
              long out = (VF[n + slab] >= 1 || z == Z - 2) ? n : n + slab;
              long in = (VF[n - slab] >= 1 || z == 1) ? n : n - slab;
              double ddz = (out == n || in == n) ? s->dhInv : gridSize;
              long right = (VF[n + 1] >= 1 || x == X - 2) ? n : n + 1;
              long left = (VF[n - 1] >= 1 || x == 1) ? n : n - 1;
              double ddx = (right == n || left == n) ? s->dhInv : gridSize;
              double N0 = (s->ws[right] - s->ws[left]) * ddx;
              double N1 = (s->ws[up] - s->ws[down]) * ddy;
              double N2 = (s->ws[out] - s->ws[in]) * ddz;
              double mag = sqrt(N0 * N0 + N1 * N1 + N2 * N2);
              if (mag > 0.0f) {
                mag = 1.0 / mag;
                N0 *= mag;
                N1 *= mag;
                N2 *= mag;
                const double* w = s->vort + 3 * n;
                double ve = s->vortEps;
                s->unitForce[3 * idx] += (N1 * w[2] - N2 * w[1]) * dh * ve * fm;
                s->unitForce[3 * idx + 1] -= (N0 * w[2] - N2 * w[0]) * dh * ve * fm;
                s->unitForce[3 * idx + 2] += (N0 * w[1] - N1 * w[0]) * dh * ve * fm;
              }
            }
          }
        } else {
          double dm = s->solidMass[n] * damp + fm;
          for (int q = 0; q < 3; q++) s->damped[3 * sidx + q] = dm;
          for (int q = 0; q < 3; q++) s->solidMv[3 * sidx + q] += fm * vn[q];
          double mg = mass * g;
          s->solidUnitForce[3 * sidx + 0] += mg * 0.0;
          s->solidUnitForce[3 * sidx + 1] += mg * -1.0;
          s->solidUnitForce[3 * sidx + 2] += mg * 0.0;
          s->solidUnitForce[3 * sidx + 1] += bu * fm * s->intensity[n];
        }
        double mi = 1.0 / mass;
        for (int q = 0; q < 3; q++) s->nzMassInv[3 * idx + q] = mi;
        energy += 0.5 * fm * (vn[0] * vn[0] + (vn[1] * vn[1] + vn[2] * vn[2]));
      }
  /* system matrix (:609-620): setFromTriplets sums duplicates in triplet
   * order, then *= dt^2 + beta dt, then += damped mass on the diagonal */
  qsort(tl.t, tl.n, sizeof(trip), trip_cmp);
  free(s->Ap);
  free(s->Aj);
  free(s->Ax);
  s->Ap = (int*)xcalloc(S3 + 1, 4);
  s->Aj = (int*)xcalloc(tl.n + S3, 4);
  s->Ax = (double*)xcalloc(tl.n + S3, 8);
  const double scale = dt * dt + rayB * dt;
  long e = 0, t = 0;
  for (long r = 0; r < S3; r++) {
    s->Ap[r] = (int)e;
    int haveDiag = 0;
    while (t < tl.n && tl.t[t].row == r) {
      int c = tl.t[t].col;
      double acc = tl.t[t].v;
      t++;
      while (t < tl.n && tl.t[t].row == r && tl.t[t].col == c) acc += tl.t[t++].v;
      if (!haveDiag && c > r) { /* coeffRef inserts a missing diagonal */
        s->Aj[e] = (int)r;
        s->Ax[e++] = 0.0 + s->damped[r];
        haveDiag = 1;
      }
      s->Aj[e] = c;
      s->Ax[e] = acc * scale;
      if (c == r) {
        s->Ax[e] += s->damped[r];
        haveDiag = 1;
      }
      e++;
    }
    if (!haveDiag) {
      s->Aj[e] = (int)r;
      s->Ax[e++] = 0.0 + s->damped[r];
    }
  }
  s->Ap[S3] = (int)e;
  s->annz = e;
  free(tl.t);
  for (long r = 0; r < S3; r++)
    for (int q = s->Ap[r]; q < s->Ap[r + 1]; q++)
      if (s->Aj[q] == r) s->sysDiag[r] = s->Ax[q];
  /* computeDivergenceConstraintRHS (:286-325) */
  const long cX = X - 1, cS = (long)(X - 1) * (Y - 1);
  for (int z = 0; z < Z - 1; z++)
    for (int y = 0; y < Y - 1; y++)
      for (int x = 0; x < X - 1; x++) {
        long c = x + y * cX + z * cS;
        double acc = 0;
        for (int i = 0; i < 8; i++) {
          long n = NIDX(x + (i & 1), y + ((i >> 1) & 1), z + ((i >> 2) & 1));
          if (s->dof[n] >= 0) continue;
          double sx = (i % 2 == 0) ? -1 : 1, sy = (i % 4 <= 1) ? -1 : 1, sz = (i < 4) ? -1 : 1;
          acc -= sx * v[3 * n];
          acc -= sy * v[3 * n + 1];
          acc -= sz * v[3 * n + 2];
        }
        s->rhs[c] = acc;
      }
  /* pcrImplicitSolve (:662-764) */
  for (long i = 0; i < S3; i++) s->solidUnitForce[i] *= dt;
  for (long i = 0; i < S3; i++) s->solidUnitForce[i] += s->solidMv[i];
  for (long i = 0; i < D; i++) s->unitForce[i] *= dt;
  for (long i = 0; i < D; i++) s->unitForce[i] += s->mv[i];
  double* w[6] = {s->tA, s->tB, s->tC, s->tD, s->tE, s->tF};
  sctx sc = {s->Ap, s->Aj, s->Ax, S3};
  int it[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
  double rr[3] = {0, 0, 0};
  cv[0] = pcr_solve(csr_mv, &sc, s->sysDiag, s->solidUnitForce, s->solidV0, S3,
                    s->p.implicit_solver_eps, s->p.cr_max_iterations, 1, w, &it[0], &rr[0]);
  for (long n = 0; n < s->total; n++) {
    int idx = s->dof[n];
    if (idx < 0) continue;
    int sidx = s->sdof[n];
    for (int q = 0; q < 3; q++)
      s->vstar[3 * idx + q] = (sidx < 0) ? s->unitForce[3 * idx + q] * s->nzMassInv[3 * idx]
                                         : s->solidV0[3 * sidx + q];
  }
  for (int z = 0; z < Z - 1; z++)
    for (int y = 0; y < Y - 1; y++)
      for (int x = 0; x < X - 1; x++) {
        long c = x + y * cX + z * cS;
        double jd = 0, jv = 0;
        for (int i = 0; i < 8; i++) {
          long n = NIDX(x + (i & 1), y + ((i >> 1) & 1), z + ((i >> 2) & 1));
          int k = s->dof[n];
          if (k < 0) continue;
          double sg[3] = {(i % 2 == 0) ? -1.0 : 1.0, (i % 4 <= 1) ? -1.0 : 1.0, (i < 4) ? -1.0 : 1.0};
          for (int q = 0; q < 3; q++) {
            jd += s->nzMassInv[3 * k + q] * 1.0;
            jv += sg[q] * s->vstar[3 * k + q];
          }
        }
        s->jdiag[c] = jd;
        s->b1[c] = jv - s->rhs[c];
      }
  pctx pc = {X, Y, Z, s->dof, s->nzMassInv, s->mid};
  cv[1] = pcr_solve(pressure_mv, &pc, s->jdiag, s->b1, s->lambda, R, s->p.div_free_solver_eps,
                    s->p.cr_max_iterations, 0, w, &it[1], &rr[1]);
  s->haveLambda = 1;
  /* b1 = -J^T lambda (dense over D, kept in tG) */
  double* jtl = s->tG;
  for (int z = 1; z < Z - 1; z++)
    for (int y = 1; y < Y - 1; y++)
      for (int x = 1; x < X - 1; x++) {
        int k = s->dof[NIDX(x, y, z)];
        double m0 = 0, m1 = 0, m2 = 0;
        for (int i = 7; i >= 0; i--) {
          int cx = x - (i & 1), cy = y - ((i >> 1) & 1), cz = z - ((i >> 2) & 1);
          double l = s->lambda[cx + cy * cX + cz * cS];
          double sx = (i % 2 == 0) ? -1 : 1, sy = (i % 4 <= 1) ? -1 : 1, sz = (i < 4) ? -1 : 1;
          m0 += sx * l;
          m1 += sy * l;
          m2 += sz * l;
        }
        jtl[3 * k] = -m0;
        jtl[3 * k + 1] = -m1;
        jtl[3 * k + 2] = -m2;
      }
  for (long n = 0; n < s->total; n++) {
    int sidx = s->sdof[n];
    if (sidx >= 0)
      for (int q = 0; q < 3; q++) s->solidB1[3 * sidx + q] = jtl[3 * s->dof[n] + q];
  }
  cv[2] = pcr_solve(csr_mv, &sc, s->sysDiag, s->solidB1, s->solidPC, S3, s->p.implicit_solver_eps,
                    s->p.cr_max_iterations, 1, w, &it[2], &rr[2]);
  for (long n = 0; n < s->total; n++) {
    int idx = s->dof[n];
    if (idx < 0) continue;
    int sidx = s->sdof[n];
    for (int q = 0; q < 3; q++) {
      s->pc[3 * idx + q] = (sidx < 0) ? jtl[3 * idx + q] * s->nzMassInv[3 * idx]
                                      : s->solidPC[3 * sidx + q];
      s->v1[3 * idx + q] = s->vstar[3 * idx + q] + s->pc[3 * idx + q];
      s->vel[3 * n + q] = s->v1[3 * idx + q];
    }
  }
  /* finalizeSolution (:828-917) */
  for (int i = 0; i < s->ns; i++) { /* DEFOR_SOLID_3D::finalizeSolution(v, dt) (:1182-1197) */
    solid_t* d = s->s[i];
    for (int z = d->zmin; z < d->zmax; z++)
      for (int y = d->ymin; y < d->ymax; y++)
        for (int x = d->xmin; x < d->xmax; x++) {
          long n = NIDX(x, y, z);
          for (int q = 0; q < 3; q++) d->vel[3 * n + q] = s->vel[3 * n + q];
        }
    d->dt = dt;
  }
  for (int i = 0; i < s->ns; i++) grid_to_particle(s, s->s[i]);
  for (int i = 0; i < s->ns; i++) particle_to_grid(s, s->s[i]);
  for (int i = 0; i < s->ns; i++) /* extendVectorField (:566-574) */
    for (int k = 0; k < 4; k++) sweep_vector_field(s, s->s[i], s->s[i]->vel);
  for (int i = 0; i < s->ns; i++) solid_finalize(s, s->s[i]);
  for (int i = 0; i < s->ns; i++) compute_solid_mass(s, s->s[i], 1);
  for (int i = 0; i < s->ns; i++) advect_mesh(s, s->s[i]);
  for (int i = 0; i < s->ns; i++) {
    compute_sdf(s, s->s[i]);
    init_particles(s, s->s[i]);
  }
  gather_solid_masses(s);
  fluid_advect(s);
  for (int i = 0; i < s->ns; i++) recover_velocity(s, s->s[i], s->vel);
  for (int x = 0; x < X; x++) {
    for (int y = 0; y < Y; y++) {
      for (int q = 0; q < 3; q++) {
        s->vel[3 * NIDX(x, y, 0) + q] = 0;
        s->vel[3 * NIDX(x, y, Z - 1) + q] = 0;
      }
    }
    for (int z = 0; z < Z; z++) {
      for (int q = 0; q < 3; q++) {
        s->vel[3 * NIDX(x, 0, z) + q] = 0;
        s->vel[3 * NIDX(x, Y - 1, z) + q] = 0;
      }
      s->intensity[NIDX(x, 0, z)] = 0;
    }
  }
  for (int y = 0; y < Y; y++)
    for (int z = 0; z < Z; z++)
      for (int q = 0; q < 3; q++) {
        s->vel[3 * NIDX(0, y, z) + q] = 0;
        s->vel[3 * NIDX(X - 1, y, z) + q] = 0;
      }
  if (rep) {
    memset(rep, 0, sizeof *rep);
    rep->dt = dt;
    rep->energy = energy;
    long np = 0;
    for (int i = 0; i < s->ns; i++) np += s->s[i]->np;
    rep->num_particles = (int)np;
    for (int k = 0; k < 3; k++) {
      rep->iterations[k] = it[k];
      rep->converged[k] = cv[k];
      rep->rel_residual[k] = rr[k];
    }
    rep->prone_to_contact = prone;
    rep->status = s->status;
  }
  return s->status;
}

/* -------------------------------------------------------- field access --- */
static int field_ptr(esfo_scene* s, int f, int si, void** p, size_t* count, size_t* eb) {
  long T = s->total;
  solid_t* d = (si >= 0 && si < s->ns) ? s->s[si] : NULL;
  *eb = 8;
  switch (f) {
    case ESF_F_VELOCITY: *p = s->vel; *count = T * 3; return 0;
    case ESF_F_INTENSITY: *p = s->intensity; *count = T; return 0;
    case ESF_F_SOLID_MASS: *p = s->solidMass; *count = T; return 0;
    case ESF_F_NODE_SOLID_VF: *p = s->nodeVF; *count = T; return 0;
    case ESF_F_DOF_MAP: *p = s->dof; *count = T; *eb = 4; return 0;
    case ESF_F_SOLID_DOF_MAP: *p = s->sdof; *count = T; *eb = 4; return 0;
    case ESF_F_PRESSURE: *p = s->lambda; *count = s->cells; return 0;
    case ESF_F_JMINVJT_DIAG: *p = s->jdiag; *count = s->cells; return 0;
    case ESF_F_DIV_RHS: *p = s->rhs; *count = s->cells; return 0;
    case ESF_F_B1: *p = s->b1; *count = s->cells; return 0;
    case ESF_F_NZ_MASS_INV: *p = s->nzMassInv; *count = 3L * s->nInterior; return 0;
    case ESF_F_VELOCITY_DT0: *p = s->vstar; *count = 3L * s->nInterior; return 0;
    case ESF_F_VELOCITY_DT1: *p = s->v1; *count = 3L * s->nInterior; return 0;
    case ESF_F_UNIT_FORCE: *p = s->unitForce; *count = 3L * s->nInterior; return 0;
    case ESF_F_SOLID_UNIT_FORCE: *p = s->solidUnitForce; *count = 3L * s->nSolid; return 0;
    case ESF_F_SOLID_VELOCITY_DT0: *p = s->solidV0; *count = 3L * s->nSolid; return 0;
    case ESF_F_SOLID_PRESSURE_CORRECTION: *p = s->solidPC; *count = 3L * s->nSolid; return 0;
    case ESF_F_DAMPED_SOLID_MASS: *p = s->damped; *count = 3L * s->nSolid; return 0;
    case ESF_F_SYSTEM_DIAG: *p = s->sysDiag; *count = 3L * s->nSolid; return 0;
    default: break;
  }
  if (!d) return ESF_ERR_INVALID_ARG;
  switch (f) {
    case ESF_F_S_U: *p = d->u; *count = T * 3; return 0;
    case ESF_F_S_X: *p = d->X; *count = T * 3; return 0;
    case ESF_F_S_VELOCITY: *p = d->vel; *count = T * 3; return 0;
    case ESF_F_S_VEC_WORKSPACE: *p = d->vws; *count = T * 3; return 0;
    case ESF_F_S_MASS: *p = d->mass; *count = T; return 0;
    case ESF_F_S_PHI: *p = d->phi; *count = T; return 0;
    case ESF_F_S_DET_FINV: *p = d->detFInv; *count = T; return 0;
    case ESF_F_S_VALID: *p = d->valid; *count = s->cells; *eb = 1; return 0;
    case ESF_F_S_QUARTER_FRACTIONS: *p = d->quarter; *count = T * 8; return 0;
    case ESF_F_S_PARTICLES: *p = d->part; *count = d->np * 10; return 0;
    case ESF_F_S_MESH_VERTICES: *p = d->verts; *count = d->nv * 3L; return 0;
    case ESF_F_S_FPINV:
      if (!d || !d->plastic) return ESF_ERR_INVALID_ARG;
      *p = d->FpInv;
      *count = 9L * d->pres[0] * d->pres[1] * d->pres[2];
      return 0;
    case ESF_F_S_FPINV_GRID:
      if (!d || !d->plastic) return ESF_ERR_INVALID_ARG;
      *p = d->pgrid;
      *count = 7;
      return 0;
    default: break;
  }
  return ESF_ERR_INVALID_ARG;
}

int esfo_field_info(const esfo_scene* s, int f, int si, size_t* count, size_t* eb) {
  if (!s || !count || !eb) return ESF_ERR_INVALID_ARG;
  if (f == ESF_F_S_BOXES) {
    if (si < 0 || si >= s->ns) return ESF_ERR_INVALID_ARG;
    *count = 12;
    *eb = 4;
    return ESF_OK;
  }
  if (f == ESF_F_SYSTEM_BLOCKS) {
    *count = (size_t)s->nSolid * 27 * 9;
    *eb = 8;
    return ESF_OK;
  }
  if (f == ESF_F_SYSTEM_MASK) {
    *count = (size_t)s->nSolid;
    *eb = 4;
    return ESF_OK;
  }
  void* p;
  return field_ptr((esfo_scene*)s, f, si, &p, count, eb);
}

int esfo_get_field(esfo_scene* s, int f, int si, void* host, size_t bytes) {
  if (!s || !host) return ESF_ERR_INVALID_ARG;
  if (f == ESF_F_S_BOXES) {
    if (si < 0 || si >= s->ns || bytes != 48) return ESF_ERR_INVALID_ARG;
    solid_t* d = s->s[si];
    int b[12] = {d->xmin, d->ymin, d->zmin, d->xmax, d->ymax, d->zmax,
                 d->tmin[0], d->tmin[1], d->tmin[2], d->tmax[0], d->tmax[1], d->tmax[2]};
    memcpy(host, b, 48);
    return ESF_OK;
  }
  if (f == ESF_F_SYSTEM_BLOCKS || f == ESF_F_SYSTEM_MASK) {
    /* re-layout the CSR rows of each solid node as 27 neighbour blocks */
    long S = s->nSolid;
    size_t need = (f == ESF_F_SYSTEM_BLOCKS) ? (size_t)S * 27 * 9 * 8 : (size_t)S * 4;
    if (bytes != need) return ESF_ERR_INVALID_ARG;
    int* node_of = (int*)xcalloc(S ? S : 1, 4);
    for (long n = 0; n < s->total; n++)
      if (s->sdof[n] >= 0) node_of[s->sdof[n]] = (int)n;
    double* blk = (f == ESF_F_SYSTEM_BLOCKS) ? (double*)host : NULL;
    int* mask = (f == ESF_F_SYSTEM_MASK) ? (int*)host : NULL;
    if (blk) memset(blk, 0, need);
    if (mask) memset(mask, 0, need);
    for (long r = 0; r < 3 * S && s->Ap; r++) {
      long a = r / 3;
      int ra = node_of[a], ax = ra % s->X, ay = (ra / s->X) % s->Y, az = ra / s->slab;
      for (int e = s->Ap[r]; e < s->Ap[r + 1]; e++) {
        long bcol = s->Aj[e] / 3;
        int rb = node_of[bcol], bx = rb % s->X, by = (rb / s->X) % s->Y, bz = rb / s->slab;
        int j = (bx - ax + 1) + 3 * (by - ay + 1) + 9 * (bz - az + 1);
        if (j < 0 || j >= 27) continue;
        if (blk) blk[(a * 27 + j) * 9 + (r % 3) * 3 + (s->Aj[e] % 3)] = s->Ax[e];
        if (mask) mask[a] |= (1 << j);
      }
    }
    free(node_of);
    return ESF_OK;
  }
  void* p;
  size_t count, eb;
  int st = field_ptr(s, f, si, &p, &count, &eb);
  if (st) return st;
  if (bytes != count * eb) return ESF_ERR_INVALID_ARG;
  if (bytes) memcpy(host, p, bytes);
  return ESF_OK;
}

int esfo_set_field(esfo_scene* s, int f, int si, const void* host, size_t bytes) {
  if (!s || !host) return ESF_ERR_INVALID_ARG;
  void* p;
  size_t count, eb;
  int st = field_ptr(s, f, si, &p, &count, &eb);
  if (st) return st;
  if (bytes != count * eb) return ESF_ERR_INVALID_ARG;
  if (f == ESF_F_PRESSURE) s->haveLambda = 1;
  if (bytes) memcpy(p, host, bytes);
  return ESF_OK;
}
