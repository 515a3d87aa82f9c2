/*
 * ORACLE -- test infrastructure only (see kqed_oracle.h).
 *
 * CPU restatement of the reference's composite kernels: linear
 * combinations of QED_kernel_L0 at derived arguments (x, y, 0, x - y,
 * y - x, -y) with index permutations, and the Gaussian M-subtractions.
 * Each function follows the reference function it names, term for term and
 * in the same order of operations; every L0 comes from the oracle's own
 * restatement (oracle_L0_one).  Only tests and the CPU baseline load this.
 *
 * Index convention: a kernel is K[rs][mu][nu][la], flat index
 * rs*64 + mu*16 + nu*4 + la; E(K, a, b, c) below reads K at the current
 * rs with the three Lorentz indices a, b, c.
 */
#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "kqed_oracle.h"

enum {
  C_ALL = 0, C_ALLM, C_ALLM2, C_CON, C_CON2, C_CONM, C_SUBM, C_SYMXY, C_SYMXY2, C_SYMXY0,
  C_SYMXY02, C_MKER, C_COUNT
};

#define E(K, a, b, c) (K)[rs * 64 + (a) * 16 + (b) * 4 + (c)]
#define LOOP                                                                                   \
  for (int rs = 0; rs < 6; rs++)                                                               \
    for (int mu = 0; mu < 4; mu++)                                                             \
      for (int nu = 0; nu < 4; nu++)                                                           \
        for (int la = 0; la < 4; la++)

static const double Z4[4] = {0, 0, 0, 0};

/* a struct Kernels block: 4 x 384; struct QED_Kernels: L0.xy, L0.yx, ... */
#define KS(P, l) ((P) + 384 * (l))
#define QK(P, l, yx) ((P) + 384 * (2 * (l) + (yx)))

static void L0(const double *a, const double *b, double *out) { oracle_L0_one(a, b, out); }

static double sq4(const double *v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3]; }

/* compute_all_kernels, src/LIBFILES/all_kernels.c:85-166 */
static void all_kernels(const double *x, const double *y, double *K)
{
  double Lx0[384], L0x[384], Ly0[384], L0y[384];
  double *Lxy = QK(K, 0, 0), *Lyx = QK(K, 0, 1);
  L0(x, y, Lxy);
  L0(y, x, Lyx);
  L0(x, Z4, Lx0);
  L0(Z4, x, L0x);
  L0(y, Z4, Ly0);
  L0(Z4, y, L0y);
  LOOP
  {
    const int i = rs * 64 + mu * 16 + nu * 4 + la;
    const double x0ml = E(Lx0, la, nu, mu), y0ml = E(Ly0, la, nu, mu);
    const double f1 = (x0ml + y0ml) / 2.;
    const double f2 = Lx0[i] + L0y[i];
    const double f4 = L0x[i] + Ly0[i];
    const double f3 = L0x[i] - L0y[i];
    QK(K, 1, 0)[i] = Lxy[i] + f1;
    QK(K, 2, 0)[i] = Lxy[i] - f2;
    QK(K, 3, 0)[i] = Lxy[i] + x0ml + f3;
    QK(K, 1, 1)[i] = Lyx[i] + f1;
    QK(K, 2, 1)[i] = Lyx[i] - f4;
    QK(K, 3, 1)[i] = Lyx[i] + y0ml - f3;
  }
}

/* The Gaussian subtraction terms of the M-kernels: e * (K[a][b][c] - m u *
   sum_alpha w_alpha K[...alpha...]) with alpha in source position `pos`. */
static double mterm(const double *K, int rs, int a, int b, int c, int pos, const double *w,
                    double e, double mu)
{
  double pf;
  if (pos == 0)
    pf = w[0] * E(K, 0, b, c) + w[1] * E(K, 1, b, c) + w[2] * E(K, 2, b, c) + w[3] * E(K, 3, b, c);
  else if (pos == 1)
    pf = w[0] * E(K, a, 0, c) + w[1] * E(K, a, 1, c) + w[2] * E(K, a, 2, c) + w[3] * E(K, a, 3, c);
  else
    pf = w[0] * E(K, a, b, 0) + w[1] * E(K, a, b, 1) + w[2] * E(K, a, b, 2) + w[3] * E(K, a, b, 3);
  return e * (E(K, a, b, c) - mu * pf);
}

/* compute_all_Mkernels (all_kernels.c:211-286) and _v2 (all_kernels.c:290-370) */
static void all_Mkernels(const double *M, const double *x, const double *y, double *K, int v2)
{
  double Lxy[384], Lyx[384], Lxmy[384], Lx0[384], L0x[384], Ly0[384], L0y[384];
  const double my[4] = {-y[0], -y[1], -y[2], -y[3]};
  L0(x, y, Lxy);
  if (v2) L0(x, my, Lxmy);
  L0(y, x, Lyx);
  L0(x, Z4, Lx0);
  L0(Z4, x, L0x);
  L0(y, Z4, Ly0);
  L0(Z4, y, L0y);
  const double xsq = sq4(x), ysq = sq4(y);
  for (int a = 0; a < 4; a++) {
    const double eX = exp(-M[a] * xsq / 2.), eY = exp(-M[a] * ysq / 2.);
    LOOP
    {
      const int i = rs * 64 + mu * 16 + nu * 4 + la;
      /* inlineXY(a) */
      const double XY = mterm(L0y, rs, mu, nu, la, 0, x, eX, M[a] * x[mu]) +
                        mterm(Lx0, rs, mu, nu, la, 1, y, eY, M[a] * y[nu]);
      if (!v2) {
        /* inlineYX(a) */
        const double YX = mterm(L0x, rs, mu, nu, la, 0, y, eY, M[a] * y[mu]) +
                          mterm(Ly0, rs, mu, nu, la, 1, x, eX, M[a] * x[nu]);
        QK(K, a, 0)[i] = Lxy[i] - XY;
        QK(K, a, 1)[i] = Lyx[i] - YX;
      } else {
        /* inlineYX2(a), inlineXMY(a) */
        const double YX2 = mterm(L0x, rs, nu, mu, la, 0, y, eY, M[a] * y[nu]) +
                           mterm(Ly0, rs, nu, mu, la, 1, x, eX, M[a] * x[mu]);
        const double XMY = -mterm(L0y, rs, mu, nu, la, 0, x, eX, M[a] * x[mu]) +
                           mterm(Lx0, rs, mu, nu, la, 1, y, eY, M[a] * y[nu]);
        QK(K, a, 0)[i] = Lxy[i] - XY + E(Lyx, nu, mu, la) - YX2;
        QK(K, a, 1)[i] = Lxmy[i] - XMY;
      }
    }
  }
}

/* the nine L0 evaluations shared by compute_con_kernels and _v2 */
struct con_set {
  double Kxy[384], Kyx[384], Kxxmy[384], Kx0[384], K0x[384], Ky0[384], K0y[384], Kxmy0[384],
      K0xmy[384];
};

static void con_eval(const double *x, const double *y, struct con_set *S)
{
  const double xmy[4] = {x[0] - y[0], x[1] - y[1], x[2] - y[2], x[3] - y[3]};
  L0(x, y, S->Kxy);
  L0(y, x, S->Kyx);
  L0(x, xmy, S->Kxxmy);
  L0(x, Z4, S->Kx0);
  L0(Z4, x, S->K0x);
  L0(y, Z4, S->Ky0);
  L0(Z4, y, S->K0y);
  L0(xmy, Z4, S->Kxmy0);
  L0(Z4, xmy, S->K0xmy);
}

/* compute_con_kernels_v2, src/LIBFILES/con_kernel.c:61-165; K = struct Kernels[3] */
static void con_kernels_v2(const double *x, const double *y, double *K)
{
  static __thread struct con_set S;
  con_eval(x, y, &S);
  double *A = K, *B = K + 1536, *C = K + 3072;
  LOOP
  {
    const int i = rs * 64 + mu * 16 + nu * 4 + la;
    const double kxy = S.Kxy[i], kyx = E(S.Kyx, nu, mu, la), kxxmy = E(S.Kxxmy, la, nu, mu);
    KS(A, 0)[i] = kxy;
    KS(B, 0)[i] = kxxmy;
    KS(C, 0)[i] = kxy + kyx - kxxmy;
    KS(A, 1)[i] = KS(A, 0)[i] + (E(S.Kx0, la, nu, mu) + E(S.Ky0, la, nu, mu)) / 2;
    KS(B, 1)[i] = KS(B, 0)[i] + (S.Kx0[i] + S.Kxmy0[i]) / 2;
    KS(C, 1)[i] = KS(A, 1)[i] - KS(B, 1)[i] + kyx + (E(S.Ky0, la, mu, nu) + E(S.Kx0, la, mu, nu)) / 2;
    KS(A, 2)[i] = KS(A, 0)[i] - (S.K0y[i] + S.Kx0[i]);
    KS(B, 2)[i] = KS(B, 0)[i] - (E(S.K0xmy, la, nu, mu) + E(S.Kx0, la, nu, mu));
    KS(C, 2)[i] = KS(A, 2)[i] - KS(B, 2)[i] + kyx - (E(S.K0x, nu, mu, la) + E(S.Ky0, nu, mu, la));
    KS(A, 3)[i] = KS(A, 0)[i] + (E(S.Kx0, la, nu, mu) + S.K0x[i] - S.K0y[i]);
    KS(B, 3)[i] = KS(B, 0)[i] + (S.Kx0[i] + E(S.K0x, la, nu, mu) - E(S.K0xmy, la, nu, mu));
    KS(C, 3)[i] = KS(A, 3)[i] - KS(B, 3)[i] + kyx +
                  (E(S.Ky0, la, mu, nu) + E(S.K0y, nu, mu, la) - E(S.K0x, nu, mu, la));
  }
}

/* compute_con_kernels, src/LIBFILES/con_kernel.c:167-254; K = struct QED_Kernels */
static void con_kernels(const double *x, const double *y, double *K)
{
  static __thread struct con_set S;
  con_eval(x, y, &S);
  LOOP
  {
    const int i = rs * 64 + mu * 16 + nu * 4 + la;
    const double l0xy = S.Kxy[i] + E(S.Kyx, nu, mu, la) - E(S.Kxxmy, la, nu, mu);
    const double l0yx = E(S.Kxxmy, la, nu, mu);
    QK(K, 0, 0)[i] = l0xy;
    QK(K, 0, 1)[i] = l0yx;
    QK(K, 1, 0)[i] = l0xy + (E(S.Kx0, la, nu, mu) + E(S.Ky0, la, nu, mu) + E(S.Kx0, la, mu, nu) +
                             E(S.Ky0, la, mu, nu) - S.Kx0[i] - S.Kxmy0[i]) / 2;
    QK(K, 1, 1)[i] = l0yx + (S.Kx0[i] + S.Kxmy0[i]) / 2;
    const double l2xy = l0xy - (S.K0y[i] + S.Kx0[i] + E(S.K0x, nu, mu, la) + E(S.Ky0, nu, mu, la) -
                                E(S.K0xmy, la, nu, mu) - E(S.Kx0, la, nu, mu));
    QK(K, 2, 0)[i] = l2xy;
    QK(K, 2, 1)[i] = l0yx - (E(S.Kx0, la, nu, mu) + E(S.K0xmy, la, nu, mu));
    QK(K, 3, 0)[i] = l2xy + (S.K0x[i] + E(S.K0y, nu, mu, la) + E(S.Ky0, la, mu, nu) -
                             E(S.K0x, la, nu, mu) + E(S.Ky0, nu, mu, la));
    QK(K, 3, 1)[i] = l0yx + (S.Kx0[i] + E(S.K0x, la, nu, mu) - E(S.K0xmy, la, nu, mu));
  }
}

/* compute_con_kernelsM_L2 (con_kernel.c:258-399, sub = 0) and
   compute_sub_kernelsM_L2 (sub_kernel.c:27-167, sub = 1); K = struct Kernels[3] */
static void conM_kernels(const double *M, const double *x, const double *y, double *K, int sub)
{
  static __thread double Kxy[384], Kyx[384], Kxxmy[384], Kx0[384], K0x[384], Ky0[384], K0y[384],
      K0xmy[384];
  const double xmy[4] = {x[0] - y[0], x[1] - y[1], x[2] - y[2], x[3] - y[3]};
  L0(x, y, Kxy);
  L0(y, x, Kyx);
  L0(x, xmy, Kxxmy);
  L0(x, Z4, Kx0);
  L0(Z4, x, K0x);
  L0(y, Z4, Ky0);
  L0(Z4, y, K0y);
  L0(Z4, xmy, K0xmy);
  const double xsq = sq4(x), ysq = sq4(y), xmysq = sq4(xmy);
  for (int m = 0; m < 4; m++) {
    const double eX = exp(-M[m] * xsq / 2.), eY = exp(-M[m] * ysq / 2.),
                 eXMY = exp(-M[m] * xmysq / 2.);
    LOOP
    {
      const int i = rs * 64 + mu * 16 + nu * 4 + la;
      const double lxy = Kxy[i] - mterm(K0y, rs, mu, nu, la, 0, x, eX, M[m] * x[mu]) -
                         mterm(Kx0, rs, mu, nu, la, 1, y, eY, M[m] * y[nu]);
      const double lyx = E(Kyx, nu, mu, la) - mterm(K0x, rs, nu, mu, la, 0, y, eY, M[m] * y[nu]) -
                         mterm(Ky0, rs, nu, mu, la, 1, x, eX, M[m] * x[mu]);
      double lxxmy;
      if (!sub)
        lxxmy = E(Kxxmy, la, nu, mu) - mterm(K0xmy, rs, la, nu, mu, 0, x, eX, M[m] * x[la]) -
                mterm(Kx0, rs, la, nu, mu, 1, xmy, eXMY, M[m] * xmy[nu]);
      else
        lxxmy = E(Kxxmy, nu, la, mu) - mterm(K0xmy, rs, nu, la, mu, 0, x, eX, M[m] * x[nu]) -
                mterm(Kx0, rs, nu, la, mu, 1, xmy, eXMY, M[m] * xmy[la]);
      KS(K, m)[i] = lxy;
      KS(K + 1536, m)[i] = lxxmy;
      KS(K + 3072, m)[i] = lxy + lyx - lxxmy;
    }
  }
}

/* compute_all_kernels_SYMXY (SYMXY.c:44-85, QED_Kernels) and _v2
   (SYMXY.c:14-40, struct Kernels) */
static void symxy(const double *x, const double *y, double *K, int v2)
{
  static __thread double W[3072];
  all_kernels(x, y, W);
  for (int l = 0; l < 4; l++) {
    double *dst = v2 ? KS(K, l) : QK(K, l, 0);
    LOOP
    {
      const int i = rs * 64 + mu * 16 + nu * 4 + la;
      dst[i] = (QK(W, l, 0)[i] + E(QK(W, l, 1), nu, mu, la)) / 2;
    }
    if (!v2) {
      double *yx = QK(K, l, 1);
      LOOP yx[rs * 64 + mu * 16 + nu * 4 + la] = E(dst, nu, mu, la);
    }
  }
}

/* compute_all_kernels_SYMXY0 (SYMXY0.c:116-211, QED_Kernels) and _v2
   (SYMXY0.c:22-112, struct Kernels) */
static void symxy0(const double *x, const double *y, double *K, int v2)
{
  static __thread double Lxy[384], Lyx[384], Lxmy_x[384], Lymx_y[384], Lx_xmy[384], Ly_ymx[384],
      Lx_0[384], L0_x[384], Ly_0[384], L0_y[384], Lxmy_0[384], L0_xmy[384];
  const double xmy[4] = {x[0] - y[0], x[1] - y[1], x[2] - y[2], x[3] - y[3]};
  const double ymx[4] = {-xmy[0], -xmy[1], -xmy[2], -xmy[3]};
  L0(x, y, Lxy);
  L0(y, x, Lyx);
  L0(xmy, x, Lxmy_x);
  L0(ymx, y, Lymx_y);
  L0(x, xmy, Lx_xmy);
  L0(y, ymx, Ly_ymx);
  L0(x, Z4, Lx_0);
  L0(Z4, x, L0_x);
  L0(y, Z4, Ly_0);
  L0(Z4, y, L0_y);
  L0(xmy, Z4, Lxmy_0);
  L0(Z4, xmy, L0_xmy);
  double *o0 = v2 ? KS(K, 0) : QK(K, 0, 0), *o1 = v2 ? KS(K, 1) : QK(K, 1, 0);
  double *o2 = v2 ? KS(K, 2) : QK(K, 2, 0), *o3 = v2 ? KS(K, 3) : QK(K, 3, 0);
  LOOP
  {
    const int i = rs * 64 + mu * 16 + nu * 4 + la;
    o0[i] = (Lxy[i] + E(Lyx, nu, mu, la) - E(Lxmy_x, nu, la, mu) - E(Lymx_y, mu, la, nu) -
             E(Lx_xmy, la, nu, mu) - E(Ly_ymx, la, mu, nu)) / 6;
    const double ApC = Lx_0[i] - E(Lx_0, la, nu, mu) + E(Ly_0, nu, mu, la) - E(Ly_0, la, mu, nu);
    o1[i] = o0[i] + (-ApC + E(Lx_0, la, mu, nu) - E(Lx_0, mu, la, nu) + E(Ly_0, la, nu, mu) -
                     E(Ly_0, nu, la, mu) + E(Lxmy_0, nu, mu, la) - Lxmy_0[i] +
                     E(Lxmy_0, nu, la, mu) - E(Lxmy_0, mu, la, nu)) / 12;
    o2[i] = o0[i] - (ApC + E(L0_x, nu, mu, la) - E(L0_x, nu, la, mu) + L0_y[i] -
                     E(L0_y, mu, la, nu) + E(Lxmy_0, mu, la, nu) - E(Lxmy_0, nu, la, mu) +
                     E(L0_xmy, la, mu, nu) - E(L0_xmy, la, nu, mu)) / 6.;
    o3[i] = o2[i] + (L0_x[i] - E(L0_x, la, nu, mu) + E(L0_y, nu, mu, la) - E(L0_y, la, mu, nu) +
                     E(L0_xmy, mu, la, nu) - E(L0_xmy, nu, la, mu)) / 6.;
  }
  if (!v2)
    for (int l = 0; l < 4; l++) {
      const double *xy = QK(K, l, 0);
      double *yx = QK(K, l, 1);
      LOOP yx[rs * 64 + mu * 16 + nu * 4 + la] = E(xy, nu, mu, la);
    }
}

/* QED_Mkernel_L2, src/LIBFILES/kernels.c:181-231 */
static void mkernel_L2(double M, const double *x, const double *y, double *K)
{
  double kt[384];
  L0(x, y, K);
  const double gX = exp(-M * sq4(x) / 2.);
  L0(Z4, y, kt);
  LOOP
  {
    const int i = rs * 64 + mu * 16 + nu * 4 + la;
    K[i] -= gX * (kt[i] - M * x[mu] * (x[0] * E(kt, 0, nu, la) + x[1] * E(kt, 1, nu, la) +
                                       x[2] * E(kt, 2, nu, la) + x[3] * E(kt, 3, nu, la)));
  }
  const double gY = exp(-M * sq4(y) / 2.);
  L0(x, Z4, kt);
  LOOP
  {
    const int i = rs * 64 + mu * 16 + nu * 4 + la;
    K[i] -= gY * (kt[i] - M * y[nu] * (y[0] * E(kt, mu, 0, la) + y[1] * E(kt, mu, 1, la) +
                                       y[2] * E(kt, mu, 2, la) + y[3] * E(kt, mu, 3, la)));
  }
}

long oracle_composite_size(int which)
{
  switch (which) {
  case C_ALL: case C_ALLM: case C_ALLM2: case C_CON: case C_SYMXY: case C_SYMXY0: return 3072;
  case C_CON2: case C_CONM: case C_SUBM: return 4608;
  case C_SYMXY2: case C_SYMXY02: return 1536;
  case C_MKER: return 384;
  default: return 0;
  }
}

static void one(int which, const double *M, const double *x, const double *y, double *out)
{
  switch (which) {
  case C_ALL: all_kernels(x, y, out); break;
  case C_ALLM: all_Mkernels(M, x, y, out, 0); break;
  case C_ALLM2: all_Mkernels(M, x, y, out, 1); break;
  case C_CON: con_kernels(x, y, out); break;
  case C_CON2: con_kernels_v2(x, y, out); break;
  case C_CONM: conM_kernels(M, x, y, out, 0); break;
  case C_SUBM: conM_kernels(M, x, y, out, 1); break;
  case C_SYMXY: symxy(x, y, out, 0); break;
  case C_SYMXY2: symxy(x, y, out, 1); break;
  case C_SYMXY0: symxy0(x, y, out, 0); break;
  case C_SYMXY02: symxy0(x, y, out, 1); break;
  case C_MKER: mkernel_L2(M[0], x, y, out); break;
  }
}

int oracle_composite(int which, const double *M, long n, const double *x, const double *y,
                     double *out, int nthreads)
{
  const long sz = oracle_composite_size(which);
  if (sz == 0) return 1;
  const int needs_m = which == C_ALLM || which == C_ALLM2 || which == C_CONM ||
                      which == C_SUBM || which == C_MKER;
  if (needs_m && !M) return 1;
  double probe[384];
  if (oracle_L0_one(Z4, Z4, probe)) return 1;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
#endif
  for (long i = 0; i < n; i++) one(which, M, x + 4 * i, y + 4 * i, out + sz * i);
  return 0;
}
