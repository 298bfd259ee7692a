// 1D rules, Lagrange basis and per-degree tables of the GPU operator (host side).
//
// FE_DGQ(p) is the Lagrange basis on the p+1 Gauss-Lobatto points of [0,1]
// (deal.II FE_DGQ, lexicographic).  The operator uses three cell rules
// (OceanDG.h:448-450): QGauss(floor(1.5p)+1) for the L_h cell integrals,
// QGaussLobatto(p+2) for the zeta mass and inner faces, QGauss(p+1) for the
// discharge mass inverse; boundary faces use QGauss(floor(1.5p)+1).
#pragma once
#include <cmath>
#include <cstring>

#include "oc_layout.h"

namespace oc {

// Gauss-Legendre on [0,1] by Newton on the Legendre recurrence.
inline void gauss_rule(int n, double *x, double *w) {
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    double pn = 0, dpn = 1;
    for (int it = 0; it < 100; ++it) {
      double a = 1, b = z;
      for (int k = 2; k <= n; ++k) {
        double c = ((2 * k - 1) * z * b - (k - 1) * a) / k;
        a = b;
        b = c;
      }
      pn = b;
      dpn = n == 1 ? 1.0 : n * (z * b - a) / (z * z - 1);
      double dz = pn / dpn;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    double a = 1, b = z;
    for (int k = 2; k <= n; ++k) {
      double c = ((2 * k - 1) * z * b - (k - 1) * a) / k;
      a = b;
      b = c;
    }
    dpn = n == 1 ? 1.0 : n * (z * b - a) / (z * z - 1);
    x[n - 1 - i] = z;
    w[n - 1 - i] = 2.0 / ((1 - z * z) * dpn * dpn);
  }
  for (int i = 0; i < n / 2; ++i) {
    double s = 0.5 * (x[n - 1 - i] - x[i]), ww = 0.5 * (w[i] + w[n - 1 - i]);
    x[i] = -s; x[n - 1 - i] = s; w[i] = ww; w[n - 1 - i] = ww;
  }
  if (n % 2) x[n / 2] = 0;
  for (int i = 0; i < n; ++i) { x[i] = 0.5 * (x[i] + 1); w[i] *= 0.5; }
}

// Gauss-Lobatto on [0,1]: Newton on (1-x^2)P'_{n-1} from Chebyshev-Lobatto nodes.
inline void lobatto_rule(int n, double *x, double *w) {
  const int m = n - 1;
  double P[16];
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * i / m);
    for (int it = 0; it < 200; ++it) {
      P[0] = 1; P[1] = z;
      for (int k = 2; k <= m; ++k) P[k] = ((2 * k - 1) * z * P[k - 1] - (k - 1) * P[k - 2]) / k;
      double dz = (z * P[m] - P[m - 1]) / (n * P[m]);
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    P[0] = 1; P[1] = z;
    for (int k = 2; k <= m; ++k) P[k] = ((2 * k - 1) * z * P[k - 1] - (k - 1) * P[k - 2]) / k;
    x[m - i] = z;
    w[m - i] = 2.0 / (m * n * P[m] * P[m]);
  }
  x[0] = -1; x[m] = 1;
  for (int i = 0; i < n / 2; ++i) {
    double s = 0.5 * (x[m - i] - x[i]), ww = 0.5 * (w[i] + w[m - i]);
    x[i] = -s; x[m - i] = s; w[i] = ww; w[m - i] = ww;
  }
  if (n % 2) x[n / 2] = 0;
  for (int i = 0; i < n; ++i) { x[i] = 0.5 * (x[i] + 1); w[i] *= 0.5; }
}

inline double lag(int n, const double *xn, int i, double x) {
  double v = 1;
  for (int j = 0; j < n; ++j)
    if (j != i) v *= (x - xn[j]) / (xn[i] - xn[j]);
  return v;
}

inline double lag_d(int n, const double *xn, int i, double x) {
  double s = 0;
  for (int k = 0; k < n; ++k) {
    if (k == i) continue;
    double v = 1 / (xn[i] - xn[k]);
    for (int j = 0; j < n; ++j)
      if (j != i && j != k) v *= (x - xn[j]) / (xn[i] - xn[j]);
    s += v;
  }
  return s;
}

inline bool invert_small(int n, const double *a, double *ai) {
  double m[OC_MAXN][2 * OC_MAXN];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 2 * n; ++j) m[i][j] = j < n ? a[i * n + j] : (j - n == i);
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(m[r][c]) > std::fabs(m[p][c])) p = r;
    if (m[p][c] == 0) return false;
    for (int j = 0; j < 2 * n; ++j) std::swap(m[c][j], m[p][j]);
    double d = m[c][c];
    for (int j = 0; j < 2 * n; ++j) m[c][j] /= d;
    for (int r = 0; r < n; ++r)
      if (r != c) {
        double f = m[r][c];
        for (int j = 0; j < 2 * n; ++j) m[r][j] -= f * m[c][j];
      }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) ai[i * n + j] = m[i][n + j];
  return true;
}

// Cyclic Jacobi eigen-decomposition of a small symmetric matrix: a = V diag(e) V^T.
inline void sym_eig(int n, const double *a_in, double *e, double *V) {
  double a[OC_MAXN * OC_MAXN];
  std::memcpy(a, a_in, sizeof(double) * n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) V[i * n + j] = i == j;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) off += a[i * n + j] * a[i * n + j];
    if (off < 1e-34) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        if (std::fabs(a[p * n + q]) < 1e-300) continue;
        double th = 0.5 * (a[q * n + q] - a[p * n + p]) / a[p * n + q];
        double t = (th >= 0 ? 1 : -1) / (std::fabs(th) + std::sqrt(th * th + 1));
        double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; ++k) {  // columns
          double akp = a[k * n + p], akq = a[k * n + q];
          a[k * n + p] = c * akp - s * akq;
          a[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows
          double apk = a[p * n + k], aqk = a[q * n + k];
          a[p * n + k] = c * apk - s * aqk;
          a[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; ++i) e[i] = a[i * n + i];
}

// Fill the tables of degree p (FP64; the FP32 copy is a cast).
inline void fill_tables(int p, int max_iter, DegTables<double> &t) {
  std::memset(&t, 0, sizeof(t));
  const int N = p + 1, Q = (3 * p) / 2 + 1, G = p + 2;
  double xN[OC_MAXN], wN[OC_MAXN], xQ[OC_MAXQ], wQ[OC_MAXQ], xG[OC_MAXF], wG[OC_MAXF];
  double xM[OC_MAXN], wM[OC_MAXN];
  lobatto_rule(N, xN, wN);
  gauss_rule(Q, xQ, wQ);
  lobatto_rule(G, xG, wG);
  gauss_rule(N, xM, wM);
  for (int q = 0; q < Q; ++q) {
    t.wQ[q] = wQ[q];
    t.xQ[q] = xQ[q];
    for (int i = 0; i < N; ++i) {
      t.BQ[q][i] = lag(N, xN, i, xQ[q]);
      t.DQ[q][i] = lag_d(N, xN, i, xQ[q]);
    }
  }
  double l1 = 0.;
  for (int q = 0; q < G; ++q) {
    t.wG[q] = wG[q];
    double s = 0.;
    for (int i = 0; i < N; ++i) {
      t.BG[q][i] = lag(N, xN, i, xG[q]);
      s += std::fabs(t.BG[q][i]);
    }
    l1 = s > l1 ? s : l1;
  }
  t.lebG = l1 * l1;  // tensor-product basis: the 2D sum factorises
  double S[OC_MAXN * OC_MAXN], Si[OC_MAXN * OC_MAXN];
  for (int q = 0; q < N; ++q) {
    t.wM[q] = wM[q];
    t.xM[q] = xM[q];
    for (int i = 0; i < N; ++i) {
      S[q * N + i] = lag(N, xN, i, xM[q]);
      t.BM[q][i] = S[q * N + i];
      t.DM[q][i] = lag_d(N, xN, i, xM[q]);
    }
  }
  invert_small(N, S, Si);
  for (int i = 0; i < N; ++i)
    for (int q = 0; q < N; ++q) t.Sinv[i][q] = Si[i * N + q];
  for (int nf = 2; nf <= OC_MAXF; ++nf) {
    double xf[OC_MAXF], wf[OC_MAXF];
    lobatto_rule(nf, xf, wf);
    for (int k = 0; k < nf; ++k) {
      t.wF[nf][k] = wf[k];
      for (int s = 0; s < 3; ++s) {
        const double par = s == 0 ? xf[k] : 0.5 * ((s - 1) + xf[k]);
        for (int i = 0; i < N; ++i) t.F[s][nf][k][i] = lag(N, xN, i, par);
      }
    }
  }
  // 1D lumped mass on GL(p+2) and the closed form of max_iter sweeps of the
  // lumped iteration on a fully wet affine cell (used by the FP32 path only):
  //   delta = (W2 (x) W2) diag(g(l_i l_j)) (W1 (x) W1) b / det,
  //   A = L^-1 M (1D), L^-1/2 M L^-1/2 = Qv diag(l) Qv^T, W1 = Qv^T L^-1/2, W2 = L^-1/2 Qv,
  //   g(mu) = sum_{k<K} (1-mu)^k.
  double M1[OC_MAXN * OC_MAXN] = {0}, L1[OC_MAXN] = {0};
  for (int q = 0; q < G; ++q)
    for (int i = 0; i < N; ++i) {
      L1[i] += wG[q] * t.BG[q][i];
      for (int j = 0; j < N; ++j) M1[i * N + j] += wG[q] * t.BG[q][i] * t.BG[q][j];
    }
  double Ms[OC_MAXN * OC_MAXN], ev[OC_MAXN], Qv[OC_MAXN * OC_MAXN];
  for (int i = 0; i < N; ++i) {
    t.lump[i] = L1[i];
    for (int j = 0; j < N; ++j) Ms[i * N + j] = M1[i * N + j] / std::sqrt(L1[i] * L1[j]);
  }
  sym_eig(N, Ms, ev, Qv);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      t.W1[i][j] = Qv[j * N + i] / std::sqrt(L1[j]);  // (Qv^T L^-1/2)[i][j]
      t.W2[i][j] = Qv[i * N + j] / std::sqrt(L1[i]);  // (L^-1/2 Qv)[i][j]
    }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const double mu = ev[i] * ev[j];
      double g = 0, pw = 1;
      for (int k = 0; k < max_iter; ++k) { g += pw; pw *= (1 - mu); }
      t.Gk[i][j] = g;
    }
}

}  // namespace oc
