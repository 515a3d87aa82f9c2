/*
 * ORACLE -- test infrastructure only (see kqed_oracle.h).
 *
 * CPU restatement of the reference's perturbative lepton-loop Pi-hat
 * (src/LIBFILES/pi_pert.c): the Dirac-trace table G8 (init_g8, :140-160),
 * the modified Bessel functions K_0..K_n (bessk, :95-137; the polynomial
 * approximations of Abramowitz & Stegun 9.8.5-9.8.8 and the upward
 * recurrence K_{j+1} = K_{j-1} + 2j/x K_j), the one-loop tensor pihat1
 * (:236-389) and its (rho, sigma)-antisymmetrised sum over the three
 * photon orderings, ipihatFermLoop_antisym (:162-198).  The loops keep the
 * reference's order of operations (dense over the G8 table).
 */
#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "kqed_oracle.h"

static int G8[65536];
static int G8_ready = 0;

/* 1/4 tr(gamma_{i0} ... gamma_{i(n-1)}) for Euclidean gammas, by moving the
   last gamma to the front through anticommutators (pi_pert.c:117-138) */
static int trace4(int n, const int *idx)
{
  if (n & 1) return 0;
  if (n == 0) return 1;
  if (n == 2) return idx[0] == idx[1];
  int red[8], acc = 0;
  for (int i = 0; i < n - 1; i++) {
    if (idx[i] != idx[n - 1]) continue;
    int k = 0;
    for (int j = 0; j < n - 1; j++)
      if (j != i) red[k++] = idx[j];
    acc += ((i & 1) ? -1 : 1) * trace4(n - 2, red);
  }
  return acc;
}

static void g8_init(void)
{
  if (G8_ready) return;
  for (int i = 0; i < 65536; i++) {
    int idx[8];
    for (int k = 0; k < 8; k++) idx[k] = (i >> (2 * (7 - k))) & 3;
    G8[i] = 4 * trace4(8, idx);
  }
  G8_ready = 1;
}

static inline int g8(int a, int b, int c, int d, int e, int f, int g, int h)
{
  return G8[((((((a * 4 + b) * 4 + c) * 4 + d) * 4 + e) * 4 + f) * 4 + g) * 4 + h];
}
/* the 6- and 4-index tables are G8 with leading zero indices (gamma_0^2 = 1) */
static inline int g6(int c, int d, int e, int f, int g, int h) { return g8(0, 0, c, d, e, f, g, h); }
static inline int g4(int e, int f, int g, int h) { return g8(0, 0, 0, 0, e, f, g, h); }

/* K_0 .. K_n at x > 0 into bv[0 .. n] (pi_pert.c:95-137) */
static void bessel_k(int n, double x, double *bv)
{
  double k0, k1;
  const double tox = 2.0 / x;
  if (x <= 2.0) {
    double y = x / 3.75;
    y *= y;
    const double i0 = 1.0 + y * (3.5156229 + y * (3.0899424 + y * (1.2067492 + y * (0.2659732 +
                      y * (0.360768e-1 + y * 0.45813e-2)))));
    const double i1 = x * (0.5 + y * (0.87890594 + y * (0.51498869 + y * (0.15084934 + y *
                      (0.2658733e-1 + y * (0.301532e-2 + y * 0.32411e-3))))));
    y = 0.25 * x * x;
    const double lg = log(x / 2.0);
    k0 = (-lg * i0) + (-0.57721566 + y * (0.42278420 + y * (0.23069756 + y * (0.3488590e-1 +
         y * (0.262698e-2 + y * (0.10750e-3 + y * 0.74e-5))))));
    k1 = (lg * i1) + (1.0 / x) * (1.0 + y * (0.15443144 + y * (-0.67278579 + y * (-0.18156897 +
         y * (-0.1919402e-1 + y * (-0.110404e-2 + y * (-0.4686e-4)))))));
  } else {
    const double e = exp(-x) / sqrt(x);
    k0 = e * (1.25331414 + tox * (-0.7832358e-1 + tox * (0.2189568e-1 + tox * (-0.1062446e-1 +
         tox * (0.587872e-2 + tox * (-0.251540e-2 + tox * 0.53208e-3))))));
    k1 = e * (1.25331414 + tox * (0.23498619 + tox * (-0.3655620e-1 + tox * (0.1504268e-1 +
         tox * (-0.780353e-2 + tox * (0.325614e-2 + tox * (-0.68245e-3)))))));
  }
  bv[0] = k0;
  bv[1] = k1;
  double km = k0, k = k1;
  for (int j = 1; j < n; j++) {
    const double kp = km + j * tox * k;
    km = k;
    bv[j + 1] = k = kp;
  }
}

static double norm4(const double *v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3]); }

/* pihat1, pi_pert.c:236-389: P[rho][mu][nu][lda][sig] (1024) and
   R[mu][nu][lda][sig] (256) */
static void pihat_one(const double *x, const double *y, double *P, double *R)
{
  const double pp = M_PI * M_PI, tpp = 2 * pp, nrm = 8.2336243479292e-07;
  const double xmy[4] = {x[0] - y[0], x[1] - y[1], x[2] - y[2], x[3] - y[3]};
  const double xn = norm4(x), yn = norm4(y), dn = norm4(xmy);
  double bx[3], by[3], bd[3];
  bessel_k(2, xn, bx); bx[1] /= xn; bx[2] /= (xn * xn);
  bessel_k(2, yn, by); by[1] /= yn; by[2] /= (yn * yn);
  bessel_k(2, dn, bd); bd[1] /= dn; bd[2] /= (dn * dn);
  double e[4], f[4], g[4], q[4];
  for (int r = 0; r < 4; r++) {
    e[r] = tpp * y[r] * by[2];
    f[r] = pp * y[r] * by[1];
    g[r] = pp * y[r] * by[0];
    q[r] = 2 * f[r];
  }
  const double p = tpp * by[0], s = tpp * by[1];
  double h[4][4], ht[4][4], ell[4][4], fhat[4][4], fv[4][4][4];
  for (int r = 0; r < 4; r++)
    for (int d = 0; d < 4; d++) {
      h[r][d] = f[r] * y[d] - (r == d ? 0.5 * p : 0.0);
      ell[r][d] = e[r] * y[d] - (r == d ? s : 0.0);
    }
  for (int r = 0; r < 4; r++)
    for (int d = 0; d < 4; d++) ht[r][d] = h[d][r];
  for (int r = 0; r < 4; r++) {
    for (int d = 0; d < 4; d++) {
      fhat[d][r] = h[r][d];
      for (int c = 0; c < 4; c++)
        fv[c][d][r] = pp * (by[2] * y[c] * y[d] * y[r] +
                            ((r == d) * y[c] - (c == r) * y[d] - (c == d) * y[r]) * by[1]);
    }
    fhat[r][r] += p;
  }
  const double b11 = bx[1] * bd[1], b12 = bx[1] * bd[2], b21 = bx[2] * bd[1], b22 = bx[2] * bd[2];
  double xab[4][4], x2[4], x3[4];
  for (int a = 0; a < 4; a++) {
    for (int b = 0; b < 4; b++) xab[a][b] = x[a] * xmy[b] * b22;
    x2[a] = x[a] * b21;
    x3[a] = xmy[a] * b12;
  }
  for (int i = 0; i < 256; i++) {
    const int sig = i / 64, mu = (i / 16) & 3, nu = (i / 4) & 3, lda = i & 3;
    double tr1 = 0.0, t1[4] = {0, 0, 0, 0};
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++) {
        for (int c = 0; c < 4; c++)
          for (int d = 0; d < 4; d++) {
            const double T = xab[a][b] * g8(a, mu, b, nu, c, sig, d, lda);
            for (int r = 0; r < 4; r++) t1[r] -= fv[c][d][r] * T;
            tr1 -= ell[c][d] * T;
          }
        const double m1 = g6(a, mu, b, nu, sig, lda) * xab[a][b];
        const double m2 = g6(a, mu, nu, b, sig, lda) * x2[a] - g6(mu, a, nu, b, sig, lda) * x3[a];
        const double m4 = g6(a, mu, nu, sig, b, lda) * x2[a] - g6(mu, a, nu, sig, b, lda) * x3[a];
        const double m6 = g6(mu, nu, a, sig, b, lda) * b11;
        for (int r = 0; r < 4; r++)
          t1[r] += -g[r] * m1 - ht[b][r] * m2 - fhat[b][r] * m4 + fv[a][b][r] * m6;
        tr1 -= p * m1;
        tr1 -= q[b] * (m2 + m4);
        tr1 += ell[a][b] * m6;
      }
    const double m = g4(mu, nu, sig, lda) * b11;
    for (int r = 0; r < 4; r++) {
      t1[r] += g[r] * m;
      P[r * 256 + mu * 64 + nu * 16 + lda * 4 + sig] = nrm * t1[r];
    }
    tr1 += p * m;
    R[mu * 64 + nu * 16 + lda * 4 + sig] = nrm * tr1;
  }
}

/* ipihatFermLoop_antisym, pi_pert.c:162-198: out[6][4][4][4] */
static void pihat_antisym(const double *x, const double *y, double *out)
{
  static __thread double P1[1024], R1[256], P2[1024], R2[256], P3[1024], R3[256];
  const double mx[4] = {-x[0], -x[1], -x[2], -x[3]};
  const double ymx[4] = {y[0] - x[0], y[1] - x[1], y[2] - x[2], y[3] - x[3]};
  pihat_one(x, y, P1, R1);
  pihat_one(ymx, mx, P2, R2);
  pihat_one(mx, ymx, P3, R3);
#define PP(P, a, b, c, d, e) (P)[(a) * 256 + (b) * 64 + (c) * 16 + (d) * 4 + (e)]
#define RR(R, b, c, d, e) (R)[(b) * 64 + (c) * 16 + (d) * 4 + (e)]
  int rs = 0;
  for (int rho = 0; rho < 4; rho++)
    for (int sig = rho + 1; sig < 4; sig++, rs++)
      for (int mu = 0; mu < 4; mu++)
        for (int nu = 0; nu < 4; nu++)
          for (int la = 0; la < 4; la++)
            out[rs * 64 + mu * 16 + nu * 4 + la] =
                0.5 * (+PP(P1, rho, mu, nu, la, sig) + PP(P2, rho, nu, la, mu, sig) +
                       x[rho] * RR(R2, nu, la, mu, sig) + PP(P3, rho, la, nu, mu, sig) +
                       x[rho] * RR(R3, la, nu, mu, sig) -
                       (+PP(P1, sig, mu, nu, la, rho) + PP(P2, sig, nu, la, mu, rho) +
                        x[sig] * RR(R2, nu, la, mu, rho) + PP(P3, sig, la, nu, mu, rho) +
                        x[sig] * RR(R3, la, nu, mu, rho)));
#undef PP
#undef RR
}

int oracle_pihat(long n, const double *x, const double *y, double *out, int nthreads)
{
  g8_init();
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
#endif
  for (long i = 0; i < n; i++) pihat_antisym(x + 4 * i, y + 4 * i, out + 384 * i);
  return 0;
}

int oracle_g8(int *out)
{
  g8_init();
  memcpy(out, G8, sizeof(G8));
  return 0;
}
