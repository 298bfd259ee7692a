/*
 * oceano oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64, CPU restatement of oceano's per-stage matrix-free DG
 * shallow-water operator: OceanoOperator::perform_stage_hydro (explicit and
 * additive Runge-Kutta variants) with all of its local kernels, the
 * transport-speed reduction behind dt, the L2 projection of initial data,
 * the velocity post-processing and the vorticity refinement indicator.
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark
 * load this library, and only as the checker.  The product never links it.
 *
 * PARITY UNPINNED: the reference is a deal.II 9.5.1 application (deal.II,
 * p4est and MPI are absent here, so it cannot be built), and it ships no test
 * suite or golden vectors for this path.  The restatement is pinned instead
 * by known-answer tests: quadrature exactness, free-stream preservation
 * (also across hanging faces), lake at rest to machine precision, global
 * mass conservation and convergence against the analytic vortex.
 *
 * Organisation is deliberately different from the GPU kernels: faces are
 * looped face-centrically (one flux per face, scattered to both sides), as
 * deal.II's MatrixFree::loop does, while the GPU is element-centric.
 *
 * Reference files followed (paths inside the oceano project):
 *   lib/include/space_discretization/OceanDG.h        local kernels, stages
 *   lib/include/deal.II_oceano/operators.h             lumped inverse mass
 *   lib/include/model/shallow_water/ShallowWater.h     pointwise model
 *   lib/include/model/shallow_water/physics/*.h        friction/wind/Coriolis
 *   lib/include/numerical_flux/LaxFriedrichsModified.h LLF mass/advective flux
 *   lib/include/numerical_flux/NumericalFluxBase.h     strong pressure flux
 *   lib/include/icbc/Icbc_ShallowWaterVortex.h         vortex exact solution
 * deal.II library semantics restated (not in the reference tree): FE_DGQ
 * Lagrange basis on Gauss-Lobatto nodes, lexicographic numbering, FESystem
 * component-blocked discharge DoFs, QGauss / QGaussLobatto rules, affine
 * MappingQ(1), FEEvaluation submit/integrate, CellwiseInverseMassMatrix.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXN 5 /* p <= 4 */
#define MAXQ 7 /* floor(1.5*4)+1 */
#define MAXF 6 /* Gauss-Lobatto p+2 for p <= 4 */
#define MAXBID 16

enum { BC_NONE = 0, BC_WALL = 1, BC_SUP_IN = 2, BC_SUP_OUT = 3,
       BC_HEIGHT_IN = 4, BC_DISCHARGE_IN = 5, BC_ABSORBING = 6 };
enum { FN_CONST = 0, FN_VORTEX = 1 };

/* ------------------------------------------------------------------ */
/* 1D rules and Lagrange basis                                         */
/* ------------------------------------------------------------------ */

/* Gauss-Legendre rule on [0,1] (deal.II QGauss<1>(n)), Newton on P_n. */
static void rule_gauss(int n, double *x, double *w)
{
  for (int i = 0; i < n; ++i) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), p0 = 1, p1 = z, dp = 1;
    for (int it = 0; it < 100; ++it) {
      p0 = 1; p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1; p1 = p2;
      }
      dp = (n == 1) ? 1.0 : n * (z * p1 - p0) / (z * z - 1);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-17) break;
    }
    p0 = 1; p1 = z;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
      p0 = p1; p1 = p2;
    }
    dp = (n == 1) ? 1.0 : n * (z * p1 - p0) / (z * z - 1);
    x[n - 1 - i] = z;
    w[n - 1 - i] = 2.0 / ((1 - z * z) * dp * dp);
  }
  for (int i = 0; i < n / 2; ++i) { /* symmetrise */
    double a = 0.5 * (x[n - 1 - i] - x[i]), b = 0.5 * (w[i] + w[n - 1 - i]);
    x[i] = -a; x[n - 1 - i] = a; w[i] = b; w[n - 1 - i] = b;
  }
  if (n % 2) x[n / 2] = 0;
  for (int i = 0; i < n; ++i) { x[i] = 0.5 * (x[i] + 1); w[i] *= 0.5; }
}

/* Gauss-Lobatto rule on [0,1] (deal.II QGaussLobatto<1>(n)), the published
 * Newton iteration on (1-x^2) P'_{n-1} started from Chebyshev-Lobatto nodes. */
static void rule_lobatto(int n, double *x, double *w)
{
  const int N = n - 1;
  double P[MAXF + 2];
  for (int i = 0; i < n; ++i) {
    double z = cos(M_PI * i / N);
    for (int it = 0; it < 200; ++it) {
      P[0] = 1; P[1] = z;
      for (int k = 2; k <= N; ++k)
        P[k] = ((2 * k - 1) * z * P[k - 1] - (k - 1) * P[k - 2]) / k;
      double dz = (z * P[N] - P[N - 1]) / (n * P[N]);
      z -= dz;
      if (fabs(dz) < 1e-17) break;
    }
    P[0] = 1; P[1] = z;
    for (int k = 2; k <= N; ++k)
      P[k] = ((2 * k - 1) * z * P[k - 1] - (k - 1) * P[k - 2]) / k;
    x[N - i] = z;
    w[N - i] = 2.0 / (N * n * P[N] * P[N]);
  }
  x[0] = -1; x[N] = 1;
  for (int i = 0; i < n / 2; ++i) {
    double a = 0.5 * (x[N - i] - x[i]), b = 0.5 * (w[i] + w[N - i]);
    x[i] = -a; x[N - i] = a; w[i] = b; w[N - i] = b;
  }
  if (n % 2) x[n / 2] = 0;
  for (int i = 0; i < n; ++i) { x[i] = 0.5 * (x[i] + 1); w[i] *= 0.5; }
}

static double lagrange(int N, const double *xn, int i, double x)
{
  double v = 1;
  for (int j = 0; j < N; ++j)
    if (j != i) v *= (x - xn[j]) / (xn[i] - xn[j]);
  return v;
}

static double lagrange_d(int N, const double *xn, int i, double x)
{
  double s = 0;
  for (int k = 0; k < N; ++k) {
    if (k == i) continue;
    double v = 1 / (xn[i] - xn[k]);
    for (int j = 0; j < N; ++j)
      if (j != i && j != k) v *= (x - xn[j]) / (xn[i] - xn[j]);
    s += v;
  }
  return s;
}

static int invert(int n, const double *a, double *ainv)
{
  double m[MAXN][2 * MAXN];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 2 * n; ++j)
      m[i][j] = j < n ? a[i * n + j] : (j - n == i ? 1.0 : 0.0);
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (fabs(m[r][c]) > fabs(m[piv][c])) piv = r;
    if (m[piv][c] == 0) return -1;
    if (piv != c)
      for (int j = 0; j < 2 * n; ++j) {
        double t = m[c][j]; m[c][j] = m[piv][j]; m[piv][j] = t;
      }
    double d = m[c][c];
    for (int j = 0; j < 2 * n; ++j) m[c][j] /= d;
    for (int r = 0; r < n; ++r)
      if (r != c) {
        double f = m[r][c];
        for (int j = 0; j < 2 * n; ++j) m[r][j] -= f * m[c][j];
      }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) ainv[i * n + j] = m[i][n + j];
  return 0;
}

/* Per-degree tables. Matrices are row-major [point*N + dof]. */
typedef struct {
  int p, N, Q, G, M;
  double xN[MAXN];
  double xQ[MAXQ], wQ[MAXQ], BQ[MAXQ * MAXN], DQ[MAXQ * MAXN];
  double xG[MAXF], wG[MAXF], BG[MAXF * MAXN];
  double xM[MAXN], wM[MAXN], BM[MAXN * MAXN], BMinv[MAXN * MAXN];
} shape_t;

static void shape_init(shape_t *s, int p, int cell_rule)
{
  double w[MAXF];
  s->p = p; s->N = p + 1; s->Q = cell_rule ? p + 1 : (int)floor(1.5 * p) + 1; s->G = p + 2;
  s->M = p + 1;
  rule_lobatto(s->N, s->xN, w);
  rule_gauss(s->Q, s->xQ, s->wQ);
  rule_lobatto(s->G, s->xG, s->wG);
  rule_gauss(s->M, s->xM, s->wM);
  for (int q = 0; q < s->Q; ++q)
    for (int i = 0; i < s->N; ++i) {
      s->BQ[q * s->N + i] = lagrange(s->N, s->xN, i, s->xQ[q]);
      s->DQ[q * s->N + i] = lagrange_d(s->N, s->xN, i, s->xQ[q]);
    }
  for (int q = 0; q < s->G; ++q)
    for (int i = 0; i < s->N; ++i) s->BG[q * s->N + i] = lagrange(s->N, s->xN, i, s->xG[q]);
  for (int q = 0; q < s->M; ++q)
    for (int i = 0; i < s->N; ++i) s->BM[q * s->N + i] = lagrange(s->N, s->xN, i, s->xM[q]);
  invert(s->N, s->BM, s->BMinv);
}

/* 2D sum factorisation: out[qy*nq+qx] = sum Ay[qy][iy] Bx[qx][ix] in[iy*ni+ix] */
static void eval2d(int ni, int nq, const double *Ay, const double *Bx, const double *in, double *out)
{
  double t[MAXN * MAXQ];
  for (int iy = 0; iy < ni; ++iy)
    for (int qx = 0; qx < nq; ++qx) {
      double s = 0;
      for (int ix = 0; ix < ni; ++ix) s += Bx[qx * ni + ix] * in[iy * ni + ix];
      t[iy * nq + qx] = s;
    }
  for (int qy = 0; qy < nq; ++qy)
    for (int qx = 0; qx < nq; ++qx) {
      double s = 0;
      for (int iy = 0; iy < ni; ++iy) s += Ay[qy * ni + iy] * t[iy * nq + qx];
      out[qy * nq + qx] = s;
    }
}

/* transpose: out[iy*ni+ix] += sum Ay[qy][iy] Bx[qx][ix] in[qy*nq+qx] */
static void integ2d(int ni, int nq, const double *Ay, const double *Bx, const double *in, double *out)
{
  double t[MAXN * MAXQ];
  for (int iy = 0; iy < ni; ++iy)
    for (int qx = 0; qx < nq; ++qx) {
      double s = 0;
      for (int qy = 0; qy < nq; ++qy) s += Ay[qy * ni + iy] * in[qy * nq + qx];
      t[iy * nq + qx] = s;
    }
  for (int iy = 0; iy < ni; ++iy)
    for (int ix = 0; ix < ni; ++ix) {
      double s = 0;
      for (int qx = 0; qx < nq; ++qx) s += Bx[qx * ni + ix] * t[iy * nq + qx];
      out[iy * ni + ix] += s;
    }
}

/* square transforms with a (n x n) matrix: out = (A (x) A) in, or transposed */
static void apply2d_sq(int n, const double *A, int transpose, const double *in, double *out)
{
  double t[MAXN * MAXN];
#define AM(r, c) (transpose ? A[(c) * n + (r)] : A[(r) * n + (c)])
  for (int iy = 0; iy < n; ++iy)
    for (int a = 0; a < n; ++a) {
      double s = 0;
      for (int ix = 0; ix < n; ++ix) s += AM(a, ix) * in[iy * n + ix];
      t[iy * n + a] = s;
    }
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < n; ++a) {
      double s = 0;
      for (int iy = 0; iy < n; ++iy) s += AM(b, iy) * t[iy * n + a];
      out[b * n + a] = s;
    }
#undef AM
}

/* ------------------------------------------------------------------ */
/* Operator state                                                      */
/* ------------------------------------------------------------------ */

typedef struct {
  double g, cu4, nu;
  int friction; /* 0 none, 1 linear, 2 manning (BottomFriction.h) */
  int max_iter; /* max_iteration_height, main.cc */
  int batch;    /* SIMD lanes per cell batch for the stop rule */
  int cell_rule; /* Gauss points per direction of the cell integrals and boundary faces
                    (n_points_1d, main.cc:216 / OceanDG.h:448): 0 floor(1.5 p) + 1, 1 p + 1 */
} params_t;

typedef struct {
  int n_cells, n_inner, n_bnd;
  int *deg;
  int64_t *off;         /* zeta offset per cell (discharge: 2*off) */
  double *jac;          /* per cell: x0,y0, J00,J01,J10,J11, Ji00,Ji01,Ji10,Ji11, det */
  int *fcm, *fcp, *fbid;
  signed char *ffm, *ffp, *fsub, *forient;
  double *fnx, *fny, *flen;
  int *fnf;             /* number of face quadrature points */
  int64_t *sdo0, *sdo1, *sdo2, *sdof, *sdob; /* static-data offsets */
  const double *sd0, *sd1, *sd2, *sdf, *sdb; /* borrowed, may be NULL = 0 */
  /* cell -> face contribution slots (face index*2 + side), CSR */
  int *slot_ptr, *slot_face;
  params_t prm;
  int bc_kind[MAXBID], bc_fn[MAXBID];
  double bc_c[MAXBID][3];
  double vortex[8]; /* h0, uoo, r0, gamma, x0, y0, corr, pexp */
  shape_t sh[MAXN]; /* index = degree */
  /* face trace tables [p_side][nf][sub+1] -> nf x N values */
  double ftab[MAXN][MAXF + 1][3][MAXF * MAXN];
  double btabQ[MAXN][MAXQ * MAXN];
  int64_t n_dofs;
  double *fbuf; /* per face side: 3 * MAXN values */
} oracle_t;

static int64_t nd_of(int p) { return (int64_t)(p + 1) * (p + 1); }

static double max_d(double a, double b) { return a < b ? b : a; } /* std::max */
static double min_d(double a, double b) { return b < a ? b : a; } /* std::min */

/* ShallowWater.h:312-320 */
static double depth(const params_t *m, double z, double zb)
{
  (void)m;
  return max_d(z + zb, 1e-12);
}

/* ShallowWater.h:322-336 (desingularised velocity) */
static void velocity(const params_t *m, double z, const double *q, double zb, double *v)
{
  const double h = depth(m, z, zb);
  const double h4 = h * h * h * h;
  const double inv = sqrt(2.) * h / sqrt(h4 + max_d(h4, m->cu4));
  v[0] = q[0] * inv;
  v[1] = q[1] * inv;
}

/* BottomFriction.h:87-137 (linear), :183-213 (Manning) */
static void friction_source(const params_t *m, const double *v, double cf, double h, double *s)
{
  if (m->friction == 1) {
    s[0] = cf * h * v[0]; s[1] = cf * h * v[1];
  } else if (m->friction == 2) {
    double inv_depth = 1. / (exp(log(h) * 0.33333333333));
    double vn = sqrt(v[0] * v[0] + v[1] * v[1]);
    double hcf = m->g * cf * cf * inv_depth * vn;
    s[0] = hcf * v[0]; s[1] = hcf * v[1];
  } else {
    s[0] = 0; s[1] = 0;
  }
}

static double friction_jacobian(const params_t *m, const double *v, double cf, double h)
{
  if (m->friction == 1) return cf;
  if (m->friction == 2) {
    double inv_depth = 1. / (exp(log(h) * 1.33333333333));
    double vn = sqrt(v[0] * v[0] + v[1] * v[1]);
    return m->g * cf * cf * inv_depth * vn;
  }
  return 0;
}

/* LaxFriedrichsModified.h:161-192 */
static double massflux(const params_t *m, double zm, double zp, const double *qm, const double *qp,
                       const double *n, double zbm, double zbp)
{
  double vm[2], vp[2];
  velocity(m, zm, qm, zbm, vm);
  velocity(m, zp, qp, zbp, vp);
  const double lm = fabs(vm[0] * n[0] + vm[1] * n[1]) + sqrt(m->g * depth(m, zm, zbm));
  const double lp = fabs(vp[0] * n[0] + vp[1] * n[1]) + sqrt(m->g * depth(m, zp, zbp));
  const double lambda = max_d(lp, lm);
  const double zbs = min_d(zbm, zbp);
  const double hm = depth(m, zm, zbs), hp = depth(m, zp, zbs);
  const double fm = (hm * vm[0]) * n[0] + (hm * vm[1]) * n[1];
  const double fp = (hp * vp[0]) * n[0] + (hp * vp[1]) * n[1];
  const double cm = max_d(zm, -zbs), cp = max_d(zp, -zbs);
  return 0.5 * (fm + fp) + 0.5 * lambda * (cm - cp);
}

/* LaxFriedrichsModified.h:200-230 */
static void advflux(const params_t *m, double zm, double zp, const double *qm, const double *qp,
                    const double *n, double zbm, double zbp, double *F)
{
  double vm[2], vp[2];
  velocity(m, zm, qm, zbm, vm);
  velocity(m, zp, qp, zbp, vp);
  const double lm = fabs(vm[0] * n[0] + vm[1] * n[1]) + sqrt(m->g * depth(m, zm, zbm));
  const double lp = fabs(vp[0] * n[0] + vp[1] * n[1]) + sqrt(m->g * depth(m, zp, zbp));
  const double lambda = max_d(lp, lm);
  const double zbs = min_d(zbm, zbp);
  const double hm = depth(m, zm, zbs), hp = depth(m, zp, zbs);
  double hum[2] = {hm * vm[0], hm * vm[1]}, hup[2] = {hp * vp[0], hp * vp[1]};
  double wm[2], wp[2]; /* advective_flux recomputes the velocity from hu */
  velocity(m, zm, hum, zbs, wm);
  velocity(m, zp, hup, zbs, wp);
  const double unm = wm[0] * n[0] + wm[1] * n[1];
  const double unp = wp[0] * n[0] + wp[1] * n[1];
  for (int e = 0; e < 2; ++e)
    F[e] = 0.5 * (hum[e] * unm + hup[e] * unp) + 0.5 * lambda * (hum[e] - hup[e]);
}

/* NumericalFluxBase.h:103-126 (centred variant) */
static void presflux(const params_t *m, double zm, double zp, const double *n, double zbm,
                     double zbp, double *P)
{
  const double zbs = min_d(zbm, zbp);
  const double hp = depth(m, zp, zbs), hm = depth(m, zm, zbs);
  const double cm = max_d(zm, -zbs), cp = max_d(zp, -zbs);
  const double s = m->g * 0.25 * (hp + hm) * (cp - cm);
  P[0] = s * n[0];
  P[1] = s * n[1];
}

/* Icbc_ShallowWaterVortex.h:139-226, regularity p=2, parameterised centre,
 * background speed, radius and strength. Component 0 is depth. */
static double vortex_H(double x)
{
  const double cosx = cos(x), cos2x = cos(2. * x), sin2x = sin(2. * x), sinx = sin(x);
  const double cosx2 = cosx * cosx, cos2x2 = cos2x * cos2x, x2 = x * x;
  return 0.091145833 * cos2x + 0.182291667 * x * sin2x +
         pow(cosx, 6) * (0.015625 * cosx2 + 0.024305556) + 0.011393229 * cos2x2 +
         0.13671875 * x2 + 0.045572917 * x * cos2x * sin2x +
         0.125 * x * pow(cosx, 5) * sinx * (cosx2 + 1.166666667);
}

static double vortex_value(const oracle_t *o, double x, double y, double t, int comp)
{
  const double h0 = o->vortex[0], uoo = o->vortex[1], r0 = o->vortex[2], Gamma = o->vortex[3];
  const double corr = 4., twoPowp = 4.; /* 2^p with p = 2 */
  const double x0 = o->vortex[4] + uoo * t, y0 = o->vortex[5];
  const double radius = sqrt((x - x0) * (x - x0) + (y - y0) * (y - y0));
  const double Hpi = corr * vortex_H(0.5 * M_PI);
  const double rho_half = 0.5 * M_PI * radius / r0;
  const double Hrho = corr * vortex_H(rho_half);
  const double c = cos(rho_half), c2 = c * c;
  const double inv_gpi = 1. / (o->prm.g * M_PI * M_PI);
  const double omega = twoPowp * Gamma * c2 * c2;
  const double num = twoPowp * Gamma * r0;
  if (comp == 0) return radius < r0 ? h0 - inv_gpi * num * num * (Hpi - Hrho) : h0;
  if (comp == 1) return radius < r0 ? uoo - (y - y0) * omega : uoo;
  if (comp == 2) return radius < r0 ? (x - x0) * omega : 0.;
  return 0.1 * y;
}

static double bc_fn_value(const oracle_t *o, int bid, double x, double y, double t, int comp)
{
  if (o->bc_fn[bid] == FN_VORTEX) return vortex_value(o, x, y, t, comp);
  return comp < 3 ? o->bc_c[bid][comp] : 0.;
}

/* ------------------------------------------------------------------ */
/* Construction                                                        */
/* ------------------------------------------------------------------ */

static const int ref_normal[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};

/* dof index of the i-th node along face f of a cell with N nodes per direction */
static int face_dof(int N, int f, int i)
{
  switch (f) {
  case 0: return i * N;
  case 1: return i * N + N - 1;
  case 2: return i;
  default: return (N - 1) * N + i;
  }
}

/* face point (reference coordinates) at face parameter s */
static void face_point(int f, double s, double *xi)
{
  switch (f) {
  case 0: xi[0] = 0; xi[1] = s; break;
  case 1: xi[0] = 1; xi[1] = s; break;
  case 2: xi[0] = s; xi[1] = 0; break;
  default: xi[0] = s; xi[1] = 1; break;
  }
}

void *oc_oracle_create(int n_cells, const int *degree, const double *vertices, int n_inner,
                       int n_bnd, const int *cell_m, const int *cell_p, const signed char *face_m,
                       const signed char *face_p, const signed char *subface,
                       const signed char *orient, const int *bid, const double *params_d,
                       const int *params_i, const int *bc_kind, const int *bc_fn,
                       const double *bc_const, const double *vortex)
{
  oracle_t *o = (oracle_t *)calloc(1, sizeof(oracle_t));
  o->n_cells = n_cells; o->n_inner = n_inner; o->n_bnd = n_bnd;
  o->prm.g = params_d[0];
  o->prm.cu4 = params_d[1] * params_d[1] * params_d[1] * params_d[1];
  o->prm.nu = params_d[2];
  o->prm.friction = params_i[0];
  o->prm.max_iter = params_i[1];
  o->prm.batch = params_i[2] > 0 ? params_i[2] : 1;
  o->prm.cell_rule = params_i[3];
  for (int b = 0; b < MAXBID; ++b) {
    o->bc_kind[b] = bc_kind ? bc_kind[b] : 0;
    o->bc_fn[b] = bc_fn ? bc_fn[b] : 0;
    for (int k = 0; k < 3; ++k) o->bc_c[b][k] = bc_const ? bc_const[3 * b + k] : 0;
  }
  for (int k = 0; k < 8; ++k) o->vortex[k] = vortex ? vortex[k] : 0;
  for (int p = 1; p < MAXN; ++p) shape_init(&o->sh[p], p, o->prm.cell_rule);
  for (int p = 1; p < MAXN; ++p) {
    for (int nf = 2; nf <= MAXF; ++nf) {
      double xf[MAXF], wf[MAXF];
      rule_lobatto(nf, xf, wf);
      for (int s = -1; s <= 1; ++s)
        for (int k = 0; k < nf; ++k) {
          double t = s < 0 ? xf[k] : 0.5 * (s + xf[k]);
          for (int i = 0; i <= p; ++i)
            o->ftab[p][nf][s + 1][k * (p + 1) + i] = lagrange(p + 1, o->sh[p].xN, i, t);
        }
    }
    for (int k = 0; k < o->sh[p].Q; ++k)
      for (int i = 0; i <= p; ++i)
        o->btabQ[p][k * (p + 1) + i] = lagrange(p + 1, o->sh[p].xN, i, o->sh[p].xQ[k]);
  }
  o->deg = (int *)malloc(sizeof(int) * n_cells);
  o->off = (int64_t *)malloc(sizeof(int64_t) * (n_cells + 1));
  o->jac = (double *)malloc(sizeof(double) * 11 * n_cells);
  o->sdo0 = (int64_t *)malloc(sizeof(int64_t) * (n_cells + 1));
  o->sdo1 = (int64_t *)malloc(sizeof(int64_t) * (n_cells + 1));
  o->sdo2 = (int64_t *)malloc(sizeof(int64_t) * (n_cells + 1));
  int64_t off = 0, s0 = 0, s1 = 0, s2 = 0;
  for (int c = 0; c < n_cells; ++c) {
    const int p = degree[c];
    o->deg[c] = p;
    o->off[c] = off; off += nd_of(p);
    o->sdo0[c] = s0; s0 += 5 * o->sh[p].Q * o->sh[p].Q;
    o->sdo1[c] = s1; s1 += (p + 2) * (p + 2);
    o->sdo2[c] = s2; s2 += 2 * (p + 1) * (p + 1);
    const double *v = vertices + 8 * c;
    double *J = o->jac + 11 * c;
    J[0] = v[0]; J[1] = v[1];
    J[2] = v[2] - v[0]; J[3] = v[4] - v[0]; /* J[d][a] = dx_d/dxi_a */
    J[4] = v[3] - v[1]; J[5] = v[5] - v[1];
    const double det = J[2] * J[5] - J[3] * J[4];
    J[6] = J[5] / det; J[7] = -J[3] / det; /* Jinv[a][d] */
    J[8] = -J[4] / det; J[9] = J[2] / det;
    J[10] = det;
  }
  o->off[n_cells] = off; o->n_dofs = off;
  o->sdo0[n_cells] = s0; o->sdo1[n_cells] = s1; o->sdo2[n_cells] = s2;
  const int nf_tot = n_inner + n_bnd;
  o->fcm = (int *)malloc(sizeof(int) * nf_tot);
  o->fcp = (int *)malloc(sizeof(int) * nf_tot);
  o->fbid = (int *)malloc(sizeof(int) * nf_tot);
  o->ffm = (signed char *)malloc(nf_tot);
  o->ffp = (signed char *)malloc(nf_tot);
  o->fsub = (signed char *)malloc(nf_tot);
  o->forient = (signed char *)malloc(nf_tot);
  o->fnx = (double *)malloc(sizeof(double) * nf_tot);
  o->fny = (double *)malloc(sizeof(double) * nf_tot);
  o->flen = (double *)malloc(sizeof(double) * nf_tot);
  o->fnf = (int *)malloc(sizeof(int) * nf_tot);
  o->sdof = (int64_t *)malloc(sizeof(int64_t) * (n_inner + 1));
  o->sdob = (int64_t *)malloc(sizeof(int64_t) * (n_bnd + 1));
  int64_t sf = 0, sb = 0;
  int *count = (int *)calloc(n_cells + 1, sizeof(int));
  for (int f = 0; f < nf_tot; ++f) {
    const int cm = cell_m[f];
    o->fcm[f] = cm;
    o->fcp[f] = f < n_inner ? cell_p[f] : -1;
    o->ffm[f] = face_m[f];
    o->ffp[f] = f < n_inner ? face_p[f] : -1;
    o->fsub[f] = f < n_inner ? subface[f] : -1;
    o->forient[f] = f < n_inner && orient ? orient[f] : 0;
    o->fbid[f] = f < n_inner ? -1 : bid[f - n_inner];
    const double *J = o->jac + 11 * cm;
    const int fm = face_m[f];
    /* normal = J^{-T} n_ref / |.| ; length = |J t_ref| */
    const double nr0 = ref_normal[fm][0], nr1 = ref_normal[fm][1];
    double nx = J[6] * nr0 + J[8] * nr1, ny = J[7] * nr0 + J[9] * nr1;
    const double nn = sqrt(nx * nx + ny * ny);
    o->fnx[f] = nx / nn; o->fny[f] = ny / nn;
    const double t0 = fm < 2 ? 0 : 1, t1 = fm < 2 ? 1 : 0;
    const double tx = J[2] * t0 + J[3] * t1, ty = J[4] * t0 + J[5] * t1;
    o->flen[f] = sqrt(tx * tx + ty * ty);
    if (f < n_inner) {
      const int pm = degree[cm], pp = degree[cell_p[f]];
      o->fnf[f] = (pm > pp ? pm : pp) + 2;
      o->sdof[f] = sf; sf += 2 * o->fnf[f];
      count[cm]++; count[cell_p[f]]++;
    } else {
      o->fnf[f] = o->sh[degree[cm]].Q;
      o->sdob[f - n_inner] = sb; sb += o->fnf[f];
      count[cm]++;
    }
  }
  o->sdof[n_inner] = sf; o->sdob[n_bnd] = sb;
  o->slot_ptr = (int *)malloc(sizeof(int) * (n_cells + 1));
  o->slot_ptr[0] = 0;
  for (int c = 0; c < n_cells; ++c) o->slot_ptr[c + 1] = o->slot_ptr[c] + count[c];
  o->slot_face = (int *)malloc(sizeof(int) * o->slot_ptr[n_cells]);
  memset(count, 0, sizeof(int) * (n_cells + 1));
  for (int f = 0; f < nf_tot; ++f) {
    const int cm = o->fcm[f];
    o->slot_face[o->slot_ptr[cm] + count[cm]++] = 2 * f;
    if (f < n_inner) {
      const int cp = o->fcp[f];
      o->slot_face[o->slot_ptr[cp] + count[cp]++] = 2 * f + 1;
    }
  }
  free(count);
  o->fbuf = (double *)calloc((size_t)nf_tot * 2 * 3 * MAXN, sizeof(double));
  return o;
}

void oc_oracle_set_static(void *h, const double *sd0, const double *sd1, const double *sd2,
                          const double *sdf, const double *sdb)
{
  oracle_t *o = (oracle_t *)h;
  o->sd0 = sd0; o->sd1 = sd1; o->sd2 = sd2; o->sdf = sdf; o->sdb = sdb;
}

void oc_oracle_destroy(void *h)
{
  oracle_t *o = (oracle_t *)h;
  if (!o) return;
  free(o->deg); free(o->off); free(o->jac); free(o->sdo0); free(o->sdo1); free(o->sdo2);
  free(o->fcm); free(o->fcp); free(o->fbid); free(o->ffm); free(o->ffp); free(o->fsub);
  free(o->forient); free(o->fnx); free(o->fny); free(o->flen); free(o->fnf); free(o->sdof);
  free(o->sdob); free(o->slot_ptr); free(o->slot_face); free(o->fbuf);
  free(o);
}

int64_t oc_oracle_n_dofs(void *h) { return ((oracle_t *)h)->n_dofs; }

/* sizes of the static-data arrays: cell0, cell1, cell2, face, boundary */
void oc_oracle_static_sizes(void *h, int64_t *out)
{
  oracle_t *o = (oracle_t *)h;
  out[0] = o->sdo0[o->n_cells]; out[1] = o->sdo1[o->n_cells]; out[2] = o->sdo2[o->n_cells];
  out[3] = o->sdof[o->n_inner]; out[4] = o->sdob[o->n_bnd];
}

static void map_point(const double *J, const double *xi, double *x)
{
  x[0] = J[0] + J[2] * xi[0] + J[3] * xi[1];
  x[1] = J[1] + J[4] * xi[0] + J[5] * xi[1];
}

/* Quadrature points of each static-data array, in storage order (OceanDG.h:497-569).
 * which: 0 cell Gauss n_q, 1 cell Gauss-Lobatto p+2, 2 cell Gauss p+1,
 * 3 inner faces (x - 1e-12 n, x + 1e-12 n per point), 4 boundary faces Gauss n_q. */
void oc_oracle_points(void *h, int which, double *xy)
{
  oracle_t *o = (oracle_t *)h;
  int64_t k = 0;
  if (which <= 2) {
    for (int c = 0; c < o->n_cells; ++c) {
      const shape_t *s = &o->sh[o->deg[c]];
      const double *J = o->jac + 11 * c;
      const int n = which == 0 ? s->Q : which == 1 ? s->G : s->M;
      const double *x1 = which == 0 ? s->xQ : which == 1 ? s->xG : s->xM;
      for (int qy = 0; qy < n; ++qy)
        for (int qx = 0; qx < n; ++qx) {
          double xi[2] = {x1[qx], x1[qy]};
          map_point(J, xi, xy + 2 * k);
          ++k;
        }
    }
  } else if (which == 3) {
    for (int f = 0; f < o->n_inner; ++f) {
      double xf[MAXF], wf[MAXF];
      rule_lobatto(o->fnf[f], xf, wf);
      const double *J = o->jac + 11 * o->fcm[f];
      for (int q = 0; q < o->fnf[f]; ++q) {
        double xi[2], x[2];
        face_point(o->ffm[f], xf[q], xi);
        map_point(J, xi, x);
        xy[2 * k] = x[0] - 1e-12 * o->fnx[f]; xy[2 * k + 1] = x[1] - 1e-12 * o->fny[f]; ++k;
        xy[2 * k] = x[0] + 1e-12 * o->fnx[f]; xy[2 * k + 1] = x[1] + 1e-12 * o->fny[f]; ++k;
      }
    }
  } else {
    for (int b = 0; b < o->n_bnd; ++b) {
      const int f = o->n_inner + b;
      const shape_t *s = &o->sh[o->deg[o->fcm[f]]];
      const double *J = o->jac + 11 * o->fcm[f];
      for (int q = 0; q < s->Q; ++q) {
        double xi[2];
        face_point(o->ffm[f], s->xQ[q], xi);
        map_point(J, xi, xy + 2 * k);
        ++k;
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* Local kernels                                                       */
/* ------------------------------------------------------------------ */

static void gather(const oracle_t *o, int c, const double *z, const double *q, double *zc,
                   double *qc)
{
  const int64_t nd = nd_of(o->deg[c]);
  if (z) memcpy(zc, z + o->off[c], sizeof(double) * nd);
  if (q) memcpy(qc, q + 2 * o->off[c], sizeof(double) * 2 * nd);
}

/* ref-gradient -> physical: g_phys[d] = sum_a Jinv[a][d] g_ref[a] */
static void grad_phys(const double *J, double gx, double gy, double *g)
{
  g[0] = J[6] * gx + J[8] * gy;
  g[1] = J[7] * gx + J[9] * gy;
}

/* F (physical vector) -> reference: Fr[a] = sum_d Jinv[a][d] F[d] */
static void vec_ref(const double *J, const double *F, double *Fr)
{
  Fr[0] = J[6] * F[0] + J[7] * F[1];
  Fr[1] = J[8] * F[0] + J[9] * F[1];
}

/* OceanDG.h:669-693: dst_zeta += int q . grad(phi) over Gauss n_q */
static void cell_height(const oracle_t *o, int c, const double *rq, double *dst)
{
  const shape_t *s = &o->sh[o->deg[c]];
  const int N = s->N, Q = s->Q, n = N * N, nq = Q * Q;
  const double *J = o->jac + 11 * c;
  double qc[2 * MAXN * MAXN], qv[2][MAXQ * MAXQ], gx[MAXQ * MAXQ], gy[MAXQ * MAXQ];
  gather(o, c, NULL, rq, NULL, qc);
  eval2d(N, Q, s->BQ, s->BQ, qc, qv[0]);
  eval2d(N, Q, s->BQ, s->BQ, qc + n, qv[1]);
  for (int k = 0; k < nq; ++k) {
    const double w = s->wQ[k % Q] * s->wQ[k / Q] * J[10];
    double F[2] = {qv[0][k], qv[1][k]}, Fr[2];
    vec_ref(J, F, Fr);
    gx[k] = Fr[0] * w; gy[k] = Fr[1] * w;
  }
  double out[MAXN * MAXN] = {0};
  integ2d(N, Q, s->BQ, s->DQ, gx, out); /* d/dxi: derivative in x */
  integ2d(N, Q, s->DQ, s->BQ, gy, out); /* d/deta: derivative in y */
  for (int i = 0; i < n; ++i) dst[o->off[c] + i] += out[i];
}

/* OceanDG.h:695-826: dst_q += int F:grad(phi) + S phi over Gauss n_q.
 * mode 0: full source (ERK); 1: non-stiff source (ARK); 2: stiff residual only. */
static void cell_discharge(const oracle_t *o, int c, const double *rz, const double *rq,
                           const double *rvel, double *dst, int mode)
{
  const params_t *m = &o->prm;
  const shape_t *s = &o->sh[o->deg[c]];
  const int N = s->N, Q = s->Q, n = N * N, nq = Q * Q;
  const double *J = o->jac + 11 * c;
  double zc[MAXN * MAXN], qc[2 * MAXN * MAXN], uc[2 * MAXN * MAXN];
  double zv[MAXQ * MAXQ], zdx[MAXQ * MAXQ], zdy[MAXQ * MAXQ], qv[2][MAXQ * MAXQ];
  double udx[2][MAXQ * MAXQ], udy[2][MAXQ * MAXQ];
  gather(o, c, rz, rq, zc, qc);
  eval2d(N, Q, s->BQ, s->BQ, zc, zv);
  eval2d(N, Q, s->BQ, s->DQ, zc, zdx);
  eval2d(N, Q, s->DQ, s->BQ, zc, zdy);
  eval2d(N, Q, s->BQ, s->BQ, qc, qv[0]);
  eval2d(N, Q, s->BQ, s->BQ, qc + n, qv[1]);
  const int visc = mode != 2 && rvel != NULL;
  if (visc) {
    memcpy(uc, rvel + 2 * o->off[c], sizeof(double) * 2 * n);
    for (int e = 0; e < 2; ++e) {
      eval2d(N, Q, s->BQ, s->DQ, uc + e * n, udx[e]);
      eval2d(N, Q, s->DQ, s->BQ, uc + e * n, udy[e]);
    }
  }
  double vals[2][MAXQ * MAXQ], gx[2][MAXQ * MAXQ], gy[2][MAXQ * MAXQ];
  const double *sd = o->sd0 ? o->sd0 + o->sdo0[c] : NULL;
  for (int k = 0; k < nq; ++k) {
    const double w = s->wQ[k % Q] * s->wQ[k / Q] * J[10];
    const double data[5] = {sd ? sd[5 * k] : 0, sd ? sd[5 * k + 1] : 0, sd ? sd[5 * k + 2] : 0,
                            sd ? sd[5 * k + 3] : 0, sd ? sd[5 * k + 4] : 0};
    const double z = zv[k], q[2] = {qv[0][k], qv[1][k]};
    double v[2];
    velocity(m, z, q, data[0], v);
    const double h = depth(m, z, data[0]);
    double S[2];
    if (mode == 2) { /* ShallowWater.h:458-472 */
      double fr[2];
      friction_source(m, v, data[1], h, fr);
      S[0] = -fr[0]; S[1] = -fr[1];
      vals[0][k] = S[0] * w; vals[1][k] = S[1] * w;
      continue;
    }
    double dz[2];
    grad_phys(J, zdx[k], zdy[k], dz);
    /* ShallowWater.h:378-403: flux[e][d] = q_e v_d - nu (gu[e][d] + gu[d][e]) + nu div I */
    double gu[2][2] = {{0, 0}, {0, 0}};
    if (visc)
      for (int e = 0; e < 2; ++e) {
        double gp[2];
        grad_phys(J, udx[e][k], udy[e][k], gp);
        gu[e][0] = h * gp[0]; gu[e][1] = h * gp[1];
      }
    const double nu = m->nu, div = gu[0][0] + gu[1][1];
    double F[2][2];
    for (int e = 0; e < 2; ++e)
      for (int d = 0; d < 2; ++d) F[e][d] = q[e] * v[d] - nu * (gu[e][d] + gu[d][e]);
    for (int e = 0; e < 2; ++e) F[e][e] += nu * div;
    /* ShallowWater.h:405-456 */
    double fr[2] = {0, 0};
    if (mode == 0) friction_source(m, v, data[1], h, fr);
    const double wind[2] = {data[2], data[3]};
    const double cor[2] = {data[4] * q[1], -data[4] * q[0]};
    for (int e = 0; e < 2; ++e)
      S[e] = -m->g * h * dz[e] - fr[e] + wind[e] + cor[e];
    for (int e = 0; e < 2; ++e) {
      double Fr[2];
      vec_ref(J, F[e], Fr);
      gx[e][k] = Fr[0] * w; gy[e][k] = Fr[1] * w;
      vals[e][k] = S[e] * w;
    }
  }
  for (int e = 0; e < 2; ++e) {
    double out[MAXN * MAXN] = {0};
    integ2d(N, Q, s->BQ, s->BQ, vals[e], out);
    if (mode != 2) {
      integ2d(N, Q, s->BQ, s->DQ, gx[e], out);
      integ2d(N, Q, s->DQ, s->BQ, gy[e], out);
    }
    for (int i = 0; i < n; ++i) dst[2 * o->off[c] + e * n + i] += out[i];
  }
}

/* Inner face (OceanDG.h:936-1050): contributions of one face to both sides,
 * into fbuf[face][side][var][i]. */
static void inner_face(oracle_t *o, int f, const double *rz, const double *rq, int want_h,
                       int want_q)
{
  const params_t *m = &o->prm;
  const int cm = o->fcm[f], cp = o->fcp[f];
  const int pm = o->deg[cm], pp = o->deg[cp], Nm = pm + 1, Np = pp + 1;
  const int nf = o->fnf[f], sub = o->fsub[f];
  double xf[MAXF], wf[MAXF];
  rule_lobatto(nf, xf, wf);
  const double *Lm = o->ftab[pm][nf][0];
  const double *Lp = o->ftab[pp][nf][sub + 1];
  double zm_d[MAXN], zp_d[MAXN], qm_d[2][MAXN], qp_d[2][MAXN];
  const int64_t nm = nd_of(pm), np = nd_of(pp);
  for (int i = 0; i < Nm; ++i) {
    const int d = face_dof(Nm, o->ffm[f], i);
    zm_d[i] = rz[o->off[cm] + d];
    qm_d[0][i] = rq[2 * o->off[cm] + d];
    qm_d[1][i] = rq[2 * o->off[cm] + nm + d];
  }
  for (int i = 0; i < Np; ++i) {
    const int d = face_dof(Np, o->ffp[f], i);
    zp_d[i] = rz[o->off[cp] + d];
    qp_d[0][i] = rq[2 * o->off[cp] + d];
    qp_d[1][i] = rq[2 * o->off[cp] + np + d];
  }
  const double n[2] = {o->fnx[f], o->fny[f]};
  const double *sd = o->sdf ? o->sdf + o->sdof[f] : NULL;
  double *bm = o->fbuf + (size_t)(2 * f) * 3 * MAXN;
  double *bp = o->fbuf + (size_t)(2 * f + 1) * 3 * MAXN;
  memset(bm, 0, sizeof(double) * 3 * MAXN);
  memset(bp, 0, sizeof(double) * 3 * MAXN);
  for (int k = 0; k < nf; ++k) {
    const int kp = o->forient[f] ? nf - 1 - k : k; /* plus-side point index */
    double zm = 0, zp = 0, qm[2] = {0, 0}, qp[2] = {0, 0};
    for (int i = 0; i < Nm; ++i) {
      const double l = Lm[k * Nm + i];
      zm += l * zm_d[i]; qm[0] += l * qm_d[0][i]; qm[1] += l * qm_d[1][i];
    }
    for (int i = 0; i < Np; ++i) {
      const double l = Lp[kp * Np + i];
      zp += l * zp_d[i]; qp[0] += l * qp_d[0][i]; qp[1] += l * qp_d[1][i];
    }
    const double zbm = sd ? sd[2 * k] : 0, zbp = sd ? sd[2 * k + 1] : 0;
    const double jxw = wf[k] * o->flen[f];
    double vm[3], vp[3];
    if (want_h) {
      const double F = massflux(m, zm, zp, qm, qp, n, zbm, zbp);
      vm[0] = -F * jxw; vp[0] = F * jxw;
    } else {
      vm[0] = vp[0] = 0;
    }
    if (want_q) {
      double Fa[2], Pm[2], Pp[2];
      advflux(m, zm, zp, qm, qp, n, zbm, zbp, Fa);
      presflux(m, zm, zp, n, zbm, zbp, Pm);
      presflux(m, zp, zm, n, zbp, zbm, Pp);
      for (int e = 0; e < 2; ++e) {
        vm[1 + e] = (-Fa[e] - Pm[e]) * jxw;
        vp[1 + e] = (Fa[e] + Pp[e]) * jxw;
      }
    } else {
      vm[1] = vm[2] = vp[1] = vp[2] = 0;
    }
    for (int v = 0; v < 3; ++v) {
      for (int i = 0; i < Nm; ++i) bm[v * MAXN + i] += Lm[k * Nm + i] * vm[v];
      for (int i = 0; i < Np; ++i) bp[v * MAXN + i] += Lp[kp * Np + i] * vp[v];
    }
  }
}

/* Boundary face (OceanDG.h:1105-1339) */
static int boundary_face(oracle_t *o, int f, double t, const double *rz, const double *rq,
                         int want_h, int want_q)
{
  const params_t *m = &o->prm;
  const int c = o->fcm[f], p = o->deg[c], N = p + 1;
  const shape_t *s = &o->sh[p];
  const int nf = s->Q;
  const double *L = o->btabQ[p];
  const int64_t nd = nd_of(p);
  double zd[MAXN], qd[2][MAXN];
  for (int i = 0; i < N; ++i) {
    const int d = face_dof(N, o->ffm[f], i);
    zd[i] = rz[o->off[c] + d];
    qd[0][i] = rq[2 * o->off[c] + d];
    qd[1][i] = rq[2 * o->off[c] + nd + d];
  }
  const double n[2] = {o->fnx[f], o->fny[f]};
  const int b = f - o->n_inner;
  const double *sd = o->sdb ? o->sdb + o->sdob[b] : NULL;
  const int bid = o->fbid[f];
  if (bid < 0 || bid >= MAXBID || o->bc_kind[bid] == BC_NONE) return -1;
  const int kind = o->bc_kind[bid];
  double *bm = o->fbuf + (size_t)(2 * f) * 3 * MAXN;
  memset(bm, 0, sizeof(double) * 3 * MAXN);
  const double *J = o->jac + 11 * c;
  for (int k = 0; k < nf; ++k) {
    double zm = 0, qm[2] = {0, 0};
    for (int i = 0; i < N; ++i) {
      zm += L[k * N + i] * zd[i];
      qm[0] += L[k * N + i] * qd[0][i];
      qm[1] += L[k * N + i] * qd[1][i];
    }
    const double zbm = sd ? sd[k] : 0;
    double xi[2], x[2];
    face_point(o->ffm[f], s->xQ[k], xi);
    map_point(J, xi, x);
    const double un = qm[0] * n[0] + qm[1] * n[1];
    double zp = zm, qp[2] = {qm[0], qm[1]};
    int at_outflow = 0;
    if (kind == BC_WALL) {
      qp[0] = qm[0] - 2. * un * n[0];
      qp[1] = qm[1] - 2. * un * n[1];
    } else if (kind == BC_SUP_IN) {
      zp = bc_fn_value(o, bid, x[0], x[1], t, 0);
      const double h = depth(m, zp, zbm);
      qp[0] = bc_fn_value(o, bid, x[0], x[1], t, 1) * h;
      qp[1] = bc_fn_value(o, bid, x[0], x[1], t, 2) * h;
    } else if (kind == BC_SUP_OUT) {
      at_outflow = 1;
    } else if (kind == BC_HEIGHT_IN) {
      zp = bc_fn_value(o, bid, x[0], x[1], t, 0);
    } else if (kind == BC_DISCHARGE_IN) {
      const double qn = bc_fn_value(o, bid, x[0], x[1], t, 1);
      qp[0] = qn * -n[0]; qp[1] = qn * -n[1];
    } else if (kind == BC_ABSORBING) {
      double zf = bc_fn_value(o, bid, x[0], x[1], t, 0);
      const double hf = depth(m, zf, zbm);
      double qf[2] = {bc_fn_value(o, bid, x[0], x[1], t, 1) * hf,
                      bc_fn_value(o, bid, x[0], x[1], t, 2) * hf};
      double v1[2], v2[2];
      velocity(m, zm, qm, zbm, v1);
      const double rp = v1[0] * n[0] + v1[1] * n[1] + 2. * sqrt(m->g * depth(m, zm, zbm));
      velocity(m, zf, qf, zbm, v2);
      const double rm = v2[0] * n[0] + v2[1] * n[1] - 2. * sqrt(m->g * depth(m, zf, zbm));
      const double cb = 0.25 * (rp - rm), hb = cb * cb / m->g, ub = 0.5 * (rp + rm);
      zp = hb - zbm;
      const double hd = depth(m, zp, zbm);
      qp[0] = ub * hd * n[0]; qp[1] = ub * hd * n[1];
    }
    const double jxw = s->wQ[k] * o->flen[f];
    double vm[3] = {0, 0, 0};
    if (want_h) vm[0] = -massflux(m, zm, zp, qm, qp, n, zbm, zbm) * jxw;
    if (want_q) {
      double Fa[2], P[2];
      advflux(m, zm, zp, qm, qp, n, zbm, zbm, Fa);
      presflux(m, zm, zp, n, zbm, zbm, P);
      Fa[0] += P[0]; Fa[1] += P[1];
      if (at_outflow && un < -1e-12) Fa[0] = Fa[1] = 0.;
      vm[1] = -Fa[0] * jxw; vm[2] = -Fa[1] * jxw;
    }
    for (int v = 0; v < 3; ++v)
      for (int i = 0; i < N; ++i) bm[v * MAXN + i] += L[k * N + i] * vm[v];
  }
  return 0;
}

/* scatter face contributions of cell c into dz / dq */
static void face_gather(const oracle_t *o, int c, double *dz, double *dq)
{
  const int p = o->deg[c], N = p + 1;
  const int64_t nd = nd_of(p);
  for (int sl = o->slot_ptr[c]; sl < o->slot_ptr[c + 1]; ++sl) {
    const int fs = o->slot_face[sl], f = fs / 2, side = fs % 2;
    const int fn = side ? o->ffp[f] : o->ffm[f];
    const double *b = o->fbuf + (size_t)fs * 3 * MAXN;
    for (int i = 0; i < N; ++i) {
      const int d = face_dof(N, fn, i);
      if (dz) dz[o->off[c] + d] += b[i];
      if (dq) {
        dq[2 * o->off[c] + d] += b[MAXN + i];
        dq[2 * o->off[c] + nd + d] += b[2 * MAXN + i];
      }
    }
  }
}

/* L_h for zeta into dz and for q into dq (mode as cell_discharge); zeroes first.
 * Returns -1 on an unknown boundary id (OceanDG.h:1199-1203). */
static int apply_Lh(oracle_t *o, double t, const double *rz, const double *rq,
                    const double *rvel, double *dz, double *dq, int qmode)
{
  const int nf_tot = o->n_inner + o->n_bnd;
  int bad = 0;
  if (dz) memset(dz, 0, sizeof(double) * o->n_dofs);
  if (dq) memset(dq, 0, sizeof(double) * 2 * o->n_dofs);
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int f = 0; f < nf_tot; ++f) {
    if (f < o->n_inner)
      inner_face(o, f, rz, rq, dz != NULL, dq != NULL);
    else
      bad |= boundary_face(o, f, t, rz, rq, dz != NULL, dq != NULL) != 0;
  }
  if (bad) return -1;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < o->n_cells; ++c) {
    if (dz) cell_height(o, c, rq, dz);
    if (dq) cell_discharge(o, c, rz, rq, rvel, dq, qmode);
    face_gather(o, c, dz, dq);
  }
  return 0;
}

/* stiff residual (OceanDG.h:795-826), cell loop only */
static void apply_stiff(oracle_t *o, const double *rz, const double *rq, double *dq)
{
  memset(dq, 0, sizeof(double) * 2 * o->n_dofs);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < o->n_cells; ++c) cell_discharge(o, c, rz, rq, NULL, dq, 2);
}

/* OceanDG.h:828-855: dst += int depth(src, zb) phi over Gauss-Lobatto p+2 */
static void cell_mass_height(const oracle_t *o, int c, const double *src, double *dst)
{
  const shape_t *s = &o->sh[o->deg[c]];
  const int N = s->N, G = s->G, n = N * N, ng = G * G;
  const double *J = o->jac + 11 * c;
  const double *zb = o->sd1 ? o->sd1 + o->sdo1[c] : NULL;
  double zc[MAXN * MAXN], zv[MAXF * MAXF], out[MAXN * MAXN] = {0};
  gather(o, c, src, NULL, zc, NULL);
  eval2d(N, G, s->BG, s->BG, zc, zv);
  for (int k = 0; k < ng; ++k)
    zv[k] = depth(&o->prm, zv[k], zb ? zb[k] : 0) * (s->wG[k % G] * s->wG[k / G] * J[10]);
  integ2d(N, G, s->BG, s->BG, zv, out);
  for (int i = 0; i < n; ++i) dst[o->off[c] + i] += out[i];
}

/* OceanDG.h:1373-1507 with operators.h:276-298, for one batch of cells */
static void inverse_mass_height_batch(const oracle_t *o, int c0, int c1, double *dst,
                                      const double *src)
{
  const params_t *m = &o->prm;
  /* epsilon lift of fully dry cells */
  for (int c = c0; c < c1; ++c) {
    const shape_t *s = &o->sh[o->deg[c]];
    const int N = s->N, G = s->G, n = N * N, ng = G * G;
    const double *zb = o->sd1 ? o->sd1 + o->sdo1[c] : NULL;
    double zc[MAXN * MAXN], zv[MAXF * MAXF];
    gather(o, c, dst, NULL, zc, NULL);
    eval2d(N, G, s->BG, s->BG, zc, zv);
    double zb_max_dry = -1.7976931348623157e308;
    int n_dry = 0;
    for (int k = 0; k < ng; ++k) {
      const double zbq = zb ? zb[k] : 0;
      if (zv[k] <= -zbq) {
        zb_max_dry = max_d(zbq, zb_max_dry);
        ++n_dry;
      }
    }
    if (n_dry == ng)
      for (int i = 0; i < n; ++i) dst[o->off[c] + i] = -zb_max_dry + 1e-09;
  }
  double norm = 1.;
  for (int k = 0; k < m->max_iter && norm > 1e-12; ++k) {
    norm = 0.;
    for (int c = c0; c < c1; ++c) {
      const shape_t *s = &o->sh[o->deg[c]];
      const int N = s->N, G = s->G, n = N * N, ng = G * G;
      const double *J = o->jac + 11 * c;
      const double *zb = o->sd1 ? o->sd1 + o->sdo1[c] : NULL;
      double rhs[MAXN * MAXN], zc[MAXN * MAXN], zv[MAXF * MAXF], mv[MAXF * MAXF];
      double mass[MAXN * MAXN] = {0};
      memcpy(rhs, src + o->off[c], sizeof(double) * n);
      gather(o, c, dst, NULL, zc, NULL);
      eval2d(N, G, s->BG, s->BG, zc, zv);
      int n_dry = 0;
      for (int q = 0; q < ng; ++q) {
        const double jxw = s->wG[q % G] * s->wG[q / G] * J[10];
        const double zbq = zb ? zb[q] : 0;
        const double msk = zv[q] <= -zbq ? 0. : 1.;
        n_dry += msk == 0.;
        mv[q] = msk * jxw;
        zv[q] = -depth(m, zv[q], zbq) * jxw;
      }
      integ2d(N, G, s->BG, s->BG, zv, rhs);
      integ2d(N, G, s->BG, s->BG, mv, mass);
      for (int i = 0; i < n; ++i) {
        const double old = zc[i];
        const double inc = n_dry < ng ? 1. / mass[i] * rhs[i] : 0.;
        const double nw = old + inc;
        dst[o->off[c] + i] = nw;
        norm += fabs(old - nw);
      }
    }
  }
}

static void inverse_mass_height(const oracle_t *o, double *dst, const double *src)
{
  const int W = o->prm.batch;
  const int nb = (o->n_cells + W - 1) / W;
#pragma omp parallel for schedule(static)
  for (int b = 0; b < nb; ++b) {
    const int c0 = b * W, c1 = c0 + W < o->n_cells ? c0 + W : o->n_cells;
    inverse_mass_height_batch(o, c0, c1, dst, src);
  }
}

/* CellwiseInverseMassMatrix on Gauss p+1: out = S^-1 diag(coef) S^-T in, per component.
 * coef == NULL -> 1/JxW. */
static void inv_mass_cell(const oracle_t *o, int c, const double *coef, const double *in,
                          double *out)
{
  const shape_t *s = &o->sh[o->deg[c]];
  const int N = s->N, n = N * N;
  const double *J = o->jac + 11 * c;
  for (int e = 0; e < 2; ++e) {
    double t[MAXN * MAXN];
    apply2d_sq(N, s->BMinv, 1, in + e * n, t);
    for (int k = 0; k < n; ++k)
      t[k] *= coef ? coef[k] : 1. / (s->wM[k % N] * s->wM[k / N] * J[10]);
    apply2d_sq(N, s->BMinv, 0, t, out + e * n);
  }
}

/* OceanoOperator::apply with its documented semantics (OceanDG.h:1658-1691;
 * the reference's own body, :1692-1727, calls functions that do not exist):
 * dst = M^-1 L_h(t, src) for zeta and q, M^-1 the exact cell inverse on Gauss
 * p+1 (CellwiseInverseMassMatrix, as for the discharge at OceanDG.h:1532-1571)
 * for all three variables.  Returns -1 on an unknown boundary id. */
int oc_oracle_apply(void *h, double t, const double *sz, const double *sq, double *dz,
                    double *dq)
{
  oracle_t *o = (oracle_t *)h;
  const int64_t nd = o->n_dofs;
  double *lz = (double *)malloc(sizeof(double) * nd);
  double *lq = (double *)malloc(sizeof(double) * 2 * nd);
  int r = apply_Lh(o, t, sz, sq, NULL, lz, lq, 0);
  if (r == 0) {
#pragma omp parallel for schedule(static)
    for (int c = 0; c < o->n_cells; ++c) {
      const shape_t *s = &o->sh[o->deg[c]];
      const int N = s->N, n = N * N;
      const double *J = o->jac + 11 * c;
      double tz[MAXN * MAXN];
      apply2d_sq(N, s->BMinv, 1, lz + o->off[c], tz);
      for (int k = 0; k < n; ++k) tz[k] *= 1. / (s->wM[k % N] * s->wM[k / N] * J[10]);
      apply2d_sq(N, s->BMinv, 0, tz, dz + o->off[c]);
      inv_mass_cell(o, c, NULL, lq + 2 * o->off[c], dq + 2 * o->off[c]);
    }
  }
  free(lz);
  free(lq);
  return r;
}

/* ------------------------------------------------------------------ */
/* Stages                                                              */
/* ------------------------------------------------------------------ */

/* OceanDG.h:1782-1912 (TIMEINTEGRATOR_EXPLICITRUNGEKUTTA).
 * ri: {zeta, q, velocity(optional)}; kz[n_stages+1], kq[n_stages+1]. */
int oc_oracle_stage_erk(void *h, int stage, int n_stages, double t, const double *f,
                        const double *rz, const double *rq, const double *rvel, double **kz,
                        double **kq, double *sol_z, double *sol_q, double *next_z,
                        double *next_q)
{
  oracle_t *o = (oracle_t *)h;
  const int64_t nd = o->n_dofs;
  if (apply_Lh(o, t, rz, rq, rvel, kz[stage + 1], kq[0], 0)) return -1;
  /* pre-lambda: kz[0] = sum_j f_j kz[j+1]; then + int depth(sol) phi */
  for (int64_t i = 0; i < nd; ++i) {
    double v = f[0] * kz[1][i];
    for (int j = 1; j < stage + 1; ++j) v += f[j] * kz[j + 1][i];
    kz[0][i] = v;
  }
#pragma omp parallel for schedule(static)
  for (int c = 0; c < o->n_cells; ++c) cell_mass_height(o, c, sol_z, kz[0]);
  if (stage == n_stages - 1) {
    inverse_mass_height(o, sol_z, kz[0]);
  } else {
    memcpy(next_z, sol_z, sizeof(double) * nd);
    inverse_mass_height(o, next_z, kz[0]);
  }
#pragma omp parallel for schedule(static)
  for (int c = 0; c < o->n_cells; ++c) {
    const int64_t n = nd_of(o->deg[c]), b = 2 * o->off[c];
    inv_mass_cell(o, c, NULL, kq[0] + b, kq[stage + 1] + b);
    for (int64_t i = b; i < b + 2 * n; ++i) {
      const double sol = sol_q[i];
      double v = sol + f[0] * kq[1][i];
      for (int j = 1; j < stage + 1; ++j) v += f[j] * kq[j + 1][i];
      if (stage == n_stages - 1) sol_q[i] = v; else next_q[i] = v;
    }
  }
  return 0;
}

/* OceanDG.h:1936-2119 (TIMEINTEGRATOR_ADDITIVERUNGEKUTTA).
 * kz[n_stages+1], kq[2*n_stages]; ft = factor_tilde_residual; fm = factor_matrix. */
int oc_oracle_stage_ark(void *h, int stage, int n_stages, double t, const double *f,
                        const double *ft, double fm, const double *rz, const double *rq,
                        const double *rvel, double **kz, double **kq, double *sol_z,
                        double *sol_q, double *next_z, double *next_q)
{
  oracle_t *o = (oracle_t *)h;
  const int64_t nd = o->n_dofs;
  const int last = stage == n_stages - 1;
  if (apply_Lh(o, t, rz, rq, rvel, kz[stage + 1], NULL, 0)) return -1;
  if (last) {
    if (apply_Lh(o, t, rz, rq, rvel, NULL, kq[2 * stage + 1], 0)) return -1;
  } else {
    if (apply_Lh(o, t, rz, rq, rvel, NULL, kq[2 * stage + 1], 1)) return -1;
    apply_stiff(o, rz, rq, kq[2 * stage + 2]);
  }
  for (int64_t i = 0; i < nd; ++i) {
    double v = f[0] * kz[1][i];
    for (int j = 1; j < stage + 1; ++j) v += f[j] * kz[j + 1][i];
    kz[0][i] = v;
  }
#pragma omp parallel for schedule(static)
  for (int c = 0; c < o->n_cells; ++c) cell_mass_height(o, c, sol_z, kz[0]);
  if (last) {
    inverse_mass_height(o, sol_z, kz[0]);
  } else {
    memcpy(next_z, sol_z, sizeof(double) * nd);
    inverse_mass_height(o, next_z, kz[0]);
  }
  if (last) {
    for (int64_t i = 0; i < 2 * nd; ++i) {
      double v = f[0] * kq[1][i];
      for (int j = 1; j < stage + 1; ++j) v += f[j] * kq[2 * j + 1][i] + f[j - 1] * kq[2 * j][i];
      kq[0][i] = v;
    }
#pragma omp parallel for schedule(static)
    for (int c = 0; c < o->n_cells; ++c) {
      const int64_t n = nd_of(o->deg[c]), b = 2 * o->off[c];
      inv_mass_cell(o, c, NULL, kq[0] + b, next_q + b);
      for (int64_t i = b; i < b + 2 * n; ++i) sol_q[i] += next_q[i];
    }
  } else {
    for (int64_t i = 0; i < 2 * nd; ++i) {
      double v = f[0] * kq[1][i] + ft[0] * kq[2][i];
      for (int j = 1; j < stage + 1; ++j) v += f[j] * kq[2 * j + 1][i] + ft[j] * kq[2 * j + 2][i];
      kq[0][i] = v;
    }
#pragma omp parallel for schedule(static)
    for (int c = 0; c < o->n_cells; ++c) {
      const shape_t *s = &o->sh[o->deg[c]];
      const int N = s->N, n = N * N;
      const double *J = o->jac + 11 * c;
      const int64_t b = 2 * o->off[c];
      /* OceanDG.h:857-880: += int q^n phi on Gauss p+1 */
      double qv[2][MAXN * MAXN];
      for (int e = 0; e < 2; ++e) {
        double out[MAXN * MAXN] = {0};
        eval2d(N, N, s->BM, s->BM, sol_q + b + e * n, qv[e]);
        for (int k = 0; k < n; ++k) qv[e][k] *= s->wM[k % N] * s->wM[k / N] * J[10];
        integ2d(N, N, s->BM, s->BM, qv[e], out);
        for (int i = 0; i < n; ++i) kq[0][b + e * n + i] += out[i];
      }
      /* OceanDG.h:1573-1645 */
      double zc[MAXN * MAXN], qc[2 * MAXN * MAXN], zv[MAXN * MAXN], q0[MAXN * MAXN],
          q1[MAXN * MAXN], coef[MAXN * MAXN];
      gather(o, c, rz, rq, zc, qc);
      eval2d(N, N, s->BM, s->BM, zc, zv);
      eval2d(N, N, s->BM, s->BM, qc, q0);
      eval2d(N, N, s->BM, s->BM, qc + n, q1);
      const double *sd = o->sd2 ? o->sd2 + o->sdo2[c] : NULL;
      for (int k = 0; k < n; ++k) {
        const double zb = sd ? sd[2 * k] : 0, cf = sd ? sd[2 * k + 1] : 0;
        const double qq[2] = {q0[k], q1[k]};
        double v[2];
        velocity(&o->prm, zv[k], qq, zb, v);
        const double jf = friction_jacobian(&o->prm, v, cf, depth(&o->prm, zv[k], zb));
        coef[k] = 1. / (s->wM[k % N] * s->wM[k / N] * J[10]);
        coef[k] *= 1. / (1. + fm * jf);
      }
      inv_mass_cell(o, c, coef, kq[0] + b, next_q + b);
    }
  }
  return 0;
}

/* OceanDG.h:2505-2580 */
double oc_oracle_transport_speed(void *h, const double *z, const double *q)
{
  oracle_t *o = (oracle_t *)h;
  double mx = 0;
#pragma omp parallel for schedule(static) reduction(max : mx)
  for (int c = 0; c < o->n_cells; ++c) {
    const shape_t *s = &o->sh[o->deg[c]];
    const int N = s->N, G = s->G, n = N * N;
    const double *J = o->jac + 11 * c;
    const double *zb = o->sd1 ? o->sd1 + o->sdo1[c] : NULL;
    double zc[MAXN * MAXN], qc[2 * MAXN * MAXN], zv[MAXF * MAXF], q0[MAXF * MAXF],
        q1[MAXF * MAXF];
    gather(o, c, z, q, zc, qc);
    eval2d(N, G, s->BG, s->BG, zc, zv);
    eval2d(N, G, s->BG, s->BG, qc, q0);
    eval2d(N, G, s->BG, s->BG, qc + n, q1);
    double local = 0;
    for (int k = 0; k < G * G; ++k) {
      const double zbq = zb ? zb[k] : 0, qq[2] = {q0[k], q1[k]};
      double v[2];
      velocity(&o->prm, zv[k], qq, zbq, v);
      /* inverse_jacobian * velocity: cs[a] = sum_d Jinv[a][d] v[d] */
      const double cs0 = J[6] * v[0] + J[7] * v[1], cs1 = J[8] * v[0] + J[9] * v[1];
      double conv = 0;
      conv = max_d(conv, fabs(cs0));
      conv = max_d(conv, fabs(cs1));
      const double sos = sqrt(o->prm.g * depth(&o->prm, zv[k], zbq));
      double ev[2] = {1., 1.};
      for (int it = 0; it < 5; ++it) {
        const double a0 = J[6] * ev[0] + J[7] * ev[1], a1 = J[8] * ev[0] + J[9] * ev[1];
        ev[0] = J[6] * a0 + J[8] * a1; /* transpose(Jinv) * a */
        ev[1] = J[7] * a0 + J[9] * a1;
        double nrm = 0;
        nrm = max_d(nrm, fabs(ev[0]));
        nrm = max_d(nrm, fabs(ev[1]));
        ev[0] /= nrm; ev[1] /= nrm;
      }
      const double j0 = J[6] * ev[0] + J[7] * ev[1], j1 = J[8] * ev[0] + J[9] * ev[1];
      const double mev = sqrt((j0 * j0 + j1 * j1) / (ev[0] * ev[0] + ev[1] * ev[1]));
      local = max_d(local, mev * sos + conv);
    }
    mx = max_d(mx, local);
  }
  return mx;
}

/* OceanDG.h:2241-2352 (project_hydro) with the vortex as the projected function;
 * fn_kind 0: vortex_value. zeta = S^-1 f0, q = S^-1 (f_{1,2} depth(f0, zb)) */
void oc_oracle_project_vortex(void *h, double t, double *z, double *q)
{
  oracle_t *o = (oracle_t *)h;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < o->n_cells; ++c) {
    const shape_t *s = &o->sh[o->deg[c]];
    const int N = s->N, n = N * N;
    const double *J = o->jac + 11 * c;
    const double *sd = o->sd2 ? o->sd2 + o->sdo2[c] : NULL;
    double fz[MAXN * MAXN], f1[MAXN * MAXN], f2[MAXN * MAXN];
    for (int k = 0; k < n; ++k) {
      double xi[2] = {s->xM[k % N], s->xM[k / N]}, x[2];
      map_point(J, xi, x);
      fz[k] = vortex_value(o, x[0], x[1], t, 0);
      const double hq = depth(&o->prm, fz[k], sd ? sd[2 * k] : 0);
      f1[k] = vortex_value(o, x[0], x[1], t, 1) * hq;
      f2[k] = vortex_value(o, x[0], x[1], t, 2) * hq;
    }
    apply2d_sq(N, s->BMinv, 0, fz, z + o->off[c]);
    apply2d_sq(N, s->BMinv, 0, f1, q + 2 * o->off[c]);
    apply2d_sq(N, s->BMinv, 0, f2, q + 2 * o->off[c] + n);
  }
}

/* OceanDG.h:2599-2662 (evaluate_velocity_field), degree >= 1 path */
void oc_oracle_velocity_field(void *h, const double *z, const double *q, double *u)
{
  oracle_t *o = (oracle_t *)h;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < o->n_cells; ++c) {
    const shape_t *s = &o->sh[o->deg[c]];
    const int N = s->N, n = N * N;
    const double *sd = o->sd2 ? o->sd2 + o->sdo2[c] : NULL;
    double zc[MAXN * MAXN], qc[2 * MAXN * MAXN], zv[MAXN * MAXN], q0[MAXN * MAXN],
        q1[MAXN * MAXN], u0[MAXN * MAXN], u1[MAXN * MAXN];
    gather(o, c, z, q, zc, qc);
    eval2d(N, N, s->BM, s->BM, zc, zv);
    eval2d(N, N, s->BM, s->BM, qc, q0);
    eval2d(N, N, s->BM, s->BM, qc + n, q1);
    for (int k = 0; k < n; ++k) {
      const double qq[2] = {q0[k], q1[k]};
      double v[2];
      velocity(&o->prm, zv[k], qq, sd ? sd[2 * k] : 0, v);
      u0[k] = v[0]; u1[k] = v[1];
    }
    apply2d_sq(N, s->BMinv, 0, u0, u + 2 * o->off[c]);
    apply2d_sq(N, s->BMinv, 0, u1, u + 2 * o->off[c] + n);
  }
}

/* hpTuner.h:247-305: per-cell max over QGauss(p_max) points of |dv/dx - du/dy| of u */
void oc_oracle_vorticity(void *h, const double *u, int n_q_1d, float *out)
{
  oracle_t *o = (oracle_t *)h;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < o->n_cells; ++c) {
    const shape_t *s = &o->sh[o->deg[c]];
    const int N = s->N, n = N * N;
    const double *J = o->jac + 11 * c;
    double xq[MAXQ + 1], wq[MAXQ + 1], B[(MAXQ + 1) * MAXN], D[(MAXQ + 1) * MAXN];
    rule_gauss(n_q_1d, xq, wq);
    for (int k = 0; k < n_q_1d; ++k)
      for (int i = 0; i < N; ++i) {
        B[k * N + i] = lagrange(N, s->xN, i, xq[k]);
        D[k * N + i] = lagrange_d(N, s->xN, i, xq[k]);
      }
    double ux[(MAXQ + 1) * (MAXQ + 1)], uy[(MAXQ + 1) * (MAXQ + 1)],
        vx[(MAXQ + 1) * (MAXQ + 1)], vy[(MAXQ + 1) * (MAXQ + 1)];
    const double *uc = u + 2 * o->off[c];
    eval2d(N, n_q_1d, B, D, uc, ux);
    eval2d(N, n_q_1d, D, B, uc, uy);
    eval2d(N, n_q_1d, B, D, uc + n, vx);
    eval2d(N, n_q_1d, D, B, uc + n, vy);
    float mv = 0.f;
    for (int k = 0; k < n_q_1d * n_q_1d; ++k) {
      double gu[2], gv[2];
      grad_phys(J, ux[k], uy[k], gu);
      grad_phys(J, vx[k], vy[k], gv);
      const float w = (float)fabs(gv[0] - gu[1]);
      mv = w > mv ? w : mv;
    }
    out[c] = mv;
  }
}

/* OceanDG.h:2380-2459 compute_errors_hydro with the travelling vortex as the
   exact solution: out[0] = sqrt(sum_cells int (depth(f0, zb) - depth(zeta_h, zb))^2),
   out[1] = sqrt(sum_cells int sum_d (f_{d+1} depth(f0, zb) - q_h,d)^2), on the
   cell Gauss rule (n_points_1d points per direction), zb from the cell static data
   (data_quadrature_cell_0, component 0); cells summed in order. */
void oc_oracle_errors_vortex(void *h, double t, const double *z, const double *q, double *out)
{
  oracle_t *o = (oracle_t *)h;
  double e0 = 0., e1 = 0.;
  for (int c = 0; c < o->n_cells; ++c) {
    const shape_t *s = &o->sh[o->deg[c]];
    const int N = s->N, n = N * N, Q = s->Q;
    const double *J = o->jac + 11 * c;
    double zv[MAXQ * MAXQ], q0[MAXQ * MAXQ], q1[MAXQ * MAXQ];
    eval2d(N, Q, s->BQ, s->BQ, z + o->off[c], zv);
    eval2d(N, Q, s->BQ, s->BQ, q + 2 * o->off[c], q0);
    eval2d(N, Q, s->BQ, s->BQ, q + 2 * o->off[c] + n, q1);
    const double *sd = o->sd0 ? o->sd0 + o->sdo0[c] : NULL;
    double c0 = 0., c1 = 0.;
    for (int qy = 0; qy < Q; ++qy)
      for (int qx = 0; qx < Q; ++qx) {
        const int k = qy * Q + qx;
        double xi[2] = {s->xQ[qx], s->xQ[qy]}, x[2];
        map_point(J, xi, x);
        const double zb = sd ? sd[5 * k] : 0.;
        const double f0 = vortex_value(o, x[0], x[1], t, 0);
        const double hq = depth(&o->prm, f0, zb);
        const double jxw = s->wQ[qx] * s->wQ[qy] * J[10];
        const double d0 = hq - depth(&o->prm, zv[k], zb);
        const double a = vortex_value(o, x[0], x[1], t, 1) * hq - q0[k];
        const double b = vortex_value(o, x[0], x[1], t, 2) * hq - q1[k];
        c0 += d0 * d0 * jxw;
        c1 += (a * a + b * b) * jxw;
      }
    e0 += c0;
    e1 += c1;
  }
  out[0] = sqrt(e0);
  out[1] = sqrt(e1);
}

/* OceanDG.h:2732-2778 prepare_for_conservative_coarsening: on every cell marked
   for the degree p -> 0 transfer, all nodal zeta values become the average of
   zeta over the wet Gauss-Lobatto (p+2) points (wet: zeta > -zb, zb from
   data_quadrature_cell_1); cells without a wet point are left unchanged. */
void oc_oracle_conservative_coarsening(void *h, const unsigned char *mark, double *z)
{
  oracle_t *o = (oracle_t *)h;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < o->n_cells; ++c) {
    if (!mark[c]) continue;
    const shape_t *s = &o->sh[o->deg[c]];
    const int N = s->N, n = N * N, G = s->G;
    const double *J = o->jac + 11 * c;
    double zv[MAXF * MAXF];
    eval2d(N, G, s->BG, s->BG, z + o->off[c], zv);
    const double *sd = o->sd1 ? o->sd1 + o->sdo1[c] : NULL;
    double area = 0., integral = 0.;
    for (int gy = 0; gy < G; ++gy)
      for (int gx = 0; gx < G; ++gx) {
        const int k = gy * G + gx;
        const double zb = sd ? sd[k] : 0.;
        const double mask = zv[k] <= -zb ? 0. : 1.;
        const double jxw = s->wG[gx] * s->wG[gy] * J[10];
        area += mask * jxw;
        integral += zv[k] * mask * jxw;
      }
    if (area > 0.) {
      const double v = integral * (1. / area);
      for (int i = 0; i < n; ++i) z[o->off[c] + i] = v;
    }
  }
}

int oc_oracle_num_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
