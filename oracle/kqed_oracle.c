/*
 * ORACLE -- test infrastructure only (see kqed_oracle.h).
 *
 * CPU restatement of the reference KQED kernel path, portable (non-AVX)
 * semantics.  Every function cites the reference file:line it follows
 * (paths relative to the reference repository root).  The arithmetic keeps
 * the reference's expressions and their evaluation order, so on an IEEE
 * machine without FMA contraction the results agree with the reference's
 * scalar build to the last bits apart from the summation order of the final
 * 384-component linear map (taken from kqed_stv_map.h).
 */
#include "kqed_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "kqed_stv_map.h"

/* ------------------------------------------------------------------ tables */

enum { QG0, QG1, QG2, QG3, QL4, QL2, dxQG0, dxQG1, dxQG2, dxQG3, dxQL4, dxQL2, d2xQG2, d2xQG3 };
/* TAYLORX rows (src/HEADERS/KQED.h:57) */
enum { TYY = 0, G0dy, G0dx, Gl2, Gl2dy, Gl21, Gl21dy, Gl3, Gl3dy, G21, G21dy, G22A, G22B,
       G22Ady, G22Bdy, G3A, G3B, G3Ady, G3Bdy, G31A, G31B, G31Ady, G31Bdy };
/* TAYLORY rows (src/HEADERS/KQED.h:60) */
enum { alpha0dx_0p = 0, alpha0_1p, alpha3_0p, beta2_1p, alpha3_1p, alpha1_0p, beta4_1p,
       alpha1_1p, alpha1dx_1p, alpha3dx_0p, alpha3dxdx_0p, beta2dx_1p, alpha3dx_1p,
       alpha1dx_0p };

typedef struct {
  int nstpx, nstpy, nffa;
  double *XX, *YY, ystp;
  int *nfx;
  float *Fm, *Fp;   /* flat; block (a,ix,iy) starts at off[(a*nstpx+ix)*nstpy+iy] */
  long *off;
  double *TX[23];
  int ny_tay;
  double *TY[14];
  int nx_tay;
} tables_t;

static tables_t G;
static int G_ready = 0;

/* CRC32C + rank-rotated pair (src/UTILS/crc32c.c:160-172) */
static uint32_t crc_tab[256];
static void crc_init(void)
{
  for (uint32_t i = 0; i < 256; i++) {
    uint32_t c = i;
    for (int k = 0; k < 8; k++) c = (c & 1u) ? (c >> 1) ^ 0x82F63B78u : (c >> 1);
    crc_tab[i] = c;
  }
}
static void ck_accum(uint32_t *a, uint32_t *b, uint32_t rank, const void *buf, size_t len)
{
  const unsigned char *p = (const unsigned char *)buf;
  uint32_t w = 0;
  while (len--) w = crc_tab[(w ^ *p++) & 0xffu] ^ (w >> 8);
  const uint32_t r29 = rank % 29u, r31 = rank % 31u;
  *a ^= r29 ? (w << r29) | (w >> (32u - r29)) : w;
  *b ^= r31 ? (w << r31) | (w >> (32u - r31)) : w;
}

static int rd(void *p, size_t sz, size_t n, FILE *f) { return fread(p, sz, n, f) != n; }

static FILE *open_table(const char *lib, const char *name)
{
  char path[4096];
  snprintf(path, sizeof(path), "%s/PRECOMP/%s", lib, name);
  FILE *f = fopen(path, "rb");
  if (!f) fprintf(stderr, "oracle: cannot open %s\n", path);
  return f;
}

/* read_ff, src/LIBFILES/io.c:42-176 */
static int load_ff(const char *lib)
{
  FILE *f = open_table(lib, "FFxy_single_cksum.bin");
  if (!f) return 1;
  int magic, n;
  uint32_t ck[2], a, b;
  if (rd(&magic, 4, 1, f) || magic != 816968) goto bad;
  if (rd(&n, 4, 1, f) || n < 2 || n > 100000) goto bad;
  G.nstpx = n;
  G.XX = malloc(sizeof(double) * n);
  if (rd(G.XX, 8, n, f) || rd(ck, 4, 2, f)) goto bad;
  a = b = 0; ck_accum(&a, &b, 0, G.XX, sizeof(double) * n);
  if (a != ck[0] || b != ck[1]) goto bad;
  if (rd(&n, 4, 1, f) || n < 2 || n > 100000) goto bad;
  G.nstpy = n;
  G.YY = malloc(sizeof(double) * n);
  if (rd(G.YY, 8, n, f) || rd(ck, 4, 2, f)) goto bad;
  a = b = 0; ck_accum(&a, &b, 0, G.YY, sizeof(double) * n);
  if (a != ck[0] || b != ck[1]) goto bad;
  G.ystp = G.YY[1] - G.YY[0];
  if (rd(&G.nffa, 4, 1, f) || G.nffa != 14) goto bad;
  {
    const long nblk = (long)G.nffa * G.nstpx * G.nstpy;
    G.off = malloc(sizeof(long) * (nblk + 1));
    G.nfx = calloc(G.nstpx, sizeof(int));
    long cap = 1 << 20, used = 0;
    G.Fm = malloc(sizeof(float) * cap);
    G.Fp = malloc(sizeof(float) * cap);
    uint32_t ma = 0, mb = 0, pa = 0, pb = 0, rank = 0;
    for (int ia = 0; ia < G.nffa; ia++) {
      if (rd(&n, 4, 1, f) || n != G.nstpx) goto bad;
      for (int ix = 0; ix < G.nstpx; ix++) {
        if (rd(&n, 4, 1, f) || n != G.nstpy) goto bad;
        for (int iy = 0; iy < G.nstpy; iy++) {
          int nf;
          if (rd(&nf, 4, 1, f) || nf < 1 || nf > 1000) goto bad;
          if (G.nfx[ix] && G.nfx[ix] != nf) goto bad; /* one length per x node */
          G.nfx[ix] = nf;
          if (used + nf > cap) {
            while (used + nf > cap) cap *= 2;
            G.Fm = realloc(G.Fm, sizeof(float) * cap);
            G.Fp = realloc(G.Fp, sizeof(float) * cap);
          }
          G.off[((long)ia * G.nstpx + ix) * G.nstpy + iy] = used;
          if (rd(G.Fm + used, 4, nf, f)) goto bad;
          ck_accum(&ma, &mb, rank, G.Fm + used, sizeof(float) * nf);
          if (rd(G.Fp + used, 4, nf, f)) goto bad;
          ck_accum(&pa, &pb, rank, G.Fp + used, sizeof(float) * nf);
          used += nf;
          rank++;
        }
      }
    }
    G.off[nblk] = used;
    uint32_t tail[4];
    if (rd(tail, 4, 4, f)) goto bad;
    if (tail[0] != ma || tail[1] != mb || tail[2] != pa || tail[3] != pb) goto bad;
  }
  fclose(f);
  return 0;
bad:
  fprintf(stderr, "oracle: malformed or corrupt FFxy table\n");
  fclose(f);
  return 1;
}

/* read_TAYLORX / read_TAYLORY, src/LIBFILES/io.c:179-289 */
static int load_taylor(const char *lib, const char *name, int nrows, int ncols, double **rows,
                       int *ncol_out)
{
  FILE *f = open_table(lib, name);
  if (!f) return 1;
  int magic, n;
  uint32_t a = 0, b = 0, ck[2];
  if (rd(&magic, 4, 1, f) || magic != 816968 || rd(&n, 4, 1, f) || n != nrows) goto bad;
  for (int i = 0; i < nrows; i++) {
    int m;
    if (rd(&m, 4, 1, f) || m != ncols) goto bad;
    rows[i] = malloc(sizeof(double) * m);
    if (rd(rows[i], 8, m, f)) goto bad;
    ck_accum(&a, &b, (uint32_t)i, rows[i], sizeof(double) * m);
  }
  if (rd(ck, 4, 2, f) || ck[0] != a || ck[1] != b) goto bad;
  *ncol_out = ncols;
  fclose(f);
  return 0;
bad:
  fprintf(stderr, "oracle: malformed or corrupt %s\n", name);
  fclose(f);
  return 1;
}

void oracle_free(void)
{
  free(G.XX); free(G.YY); free(G.nfx); free(G.Fm); free(G.Fp); free(G.off);
  for (int i = 0; i < 23; i++) free(G.TX[i]);
  for (int i = 0; i < 14; i++) free(G.TY[i]);
  memset(&G, 0, sizeof(G));
  G_ready = 0;
}

int oracle_load(const char *lib_path)
{
  if (G_ready) oracle_free();
  crc_init();
  memset(&G, 0, sizeof(G));
  if (load_ff(lib_path) || load_taylor(lib_path, "taylorx_cksum.bin", 23, 810, G.TX, &G.ny_tay) ||
      load_taylor(lib_path, "taylory_cksum.bin", 14, 100, G.TY, &G.nx_tay)) {
    oracle_free();
    return 1;
  }
  G_ready = 1;
  return 0;
}

int oracle_grid(int *nstpx, int *nstpy, double *xlo, double *xhi, double *ylo, double *yhi)
{
  if (!G_ready) return 1;
  *nstpx = G.nstpx; *nstpy = G.nstpy;
  *xlo = G.XX[0]; *xhi = G.XX[G.nstpx - 1];
  *ylo = G.YY[0]; *yhi = G.YY[G.nstpy - 1];
  return 0;
}

static inline const float *FM(int a, int ix, int iy)
{
  return G.Fm + G.off[((long)a * G.nstpx + ix) * G.nstpy + iy];
}
static inline const float *FP(int a, int ix, int iy)
{
  return G.Fp + G.off[((long)a * G.nstpx + ix) * G.nstpy + iy];
}

/* ------------------------------------------------------- interpolation */

typedef struct { double A, B, C1, C2, D, lA; int idx; } herm_t;

typedef struct {
  double x, cb, y, xsq, ysq, xdoty, cborig, yorig, xmysq, xmy;
  int flag2;
  herm_t hx, hy;
} inv_t;

static inline double lerp(double a, double t1, double t2) { return a * t1 + (1.0 - a) * t2; }

static inline double dot4(const double *a, const double *b)
{
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
}

/* bsrch, src/LIBFILES/getff-new.c:199-210 (iterative form of the same bisection) */
static int bsrch(const double *arr, double t, int lo, int hi)
{
  while (hi - lo >= 2) {
    const int mid = (hi + lo) / 2;
    if (arr[mid] > t) hi = mid;
    else lo = mid;
  }
  return lo;
}

/* precompute_INVx / precompute_INV, getff-new.c:30-47 and src/LIBFILES/simd.c:10-27 */
static void herm(herm_t *h, double y, double y1, double y2, int idx)
{
  h->idx = idx;
  const double dy = y1 - y2, ymy1 = y - y1, ymy2 = y - y2;
  const double ym2sq = ymy2 * ymy2, ym1sq = ymy1 * ymy1;
  h->A = -(ym2sq) * (2 * y - 3 * y1 + y2);
  h->B = (ym1sq) * (2 * y + y1 - 3 * y2);
  h->C1 = (ymy1) * (ym2sq)*dy;
  h->C2 = (ym1sq) * (ymy2)*dy;
  h->D = 1. / (dy * dy * dy);
  h->lA = (y2 - y) / (y2 - y1);
}

/* interpol4, getff-new.c:58-66 */
static inline double hermite_pre(const herm_t *h, double f1, double f2, double g1, double g2)
{
  return (f1 * h->A + f2 * h->B + g1 * h->C1 + g2 * h->C2) * h->D;
}

/* interpol3, getff-new.c:13-26 */
static inline double hermite_y(double y, double y1, double y2, double dy, double f1, double f2,
                               double g1, double g2)
{
  return ((-f1 * (y - y2) * (y - y2) * (2 * y - 3 * y1 + y2) +
           (y - y1) * (f2 * (y - y1) * (2 * y + y1 - 3 * y2) +
                       (y - y2) * dy * (g1 * y + g2 * y - g2 * y1 - g1 * y2))) /
          (dy * dy * dy));
}

/* Clenshaw sums of U_k and its first three derivatives, src/LIBFILES/cheby.c:13-91 */
static double cheb0(int nk, double x, const double *co)
{
  double ya = 0.0, yb = 0.0, t;
  const double twox = 2.0 * x;
  for (int j = nk - 1; j > 0; j--) { t = yb; yb = twox * yb - ya + co[j]; ya = t; }
  return (-ya + twox * yb + co[0]);
}
static double cheb1(int nk, double x, const double *co)
{
  double ya = 0.0, yb = 0.0, t;
  const double twox = 2.0 * x;
  for (int j = nk - 1; j > 0; j--) {
    t = yb;
    yb = twox * (j + 1) * yb / j - (j + 3) * ya / (j + 1) + co[j];
    ya = t;
  }
  return (2.0 * yb);
}
static double cheb2(int nk, double x, const double *co)
{
  double ya = 0.0, yb = 0.0, t;
  const double twox = 2.0 * x;
  for (int j = nk - 1; j > 1; j--) {
    t = yb;
    yb = twox * (j + 1) * yb / (j - 1);
    yb -= (j + 4) * ya / j;
    yb += co[j];
    ya = t;
  }
  return 8 * yb;
}
static double cheb3(int nk, double x, const double *co)
{
  double ya = 0.0, yb = 0.0, t;
  const double twox = 2.0 * x;
  for (int j = nk - 1; j > 2; j--) {
    t = yb;
    yb = twox * (j + 1) * yb / (j - 2) - (j + 5) * ya / (j - 1) + co[j];
    ya = t;
  }
  return 48 * yb;
}
static double chebd(int order, int nk, double x, const double *co)
{
  switch (order) {
  case 0: return cheb0(nk, x, co);
  case 1: return cheb1(nk, x, co);
  case 2: return cheb2(nk, x, co);
  case 3: return cheb3(nk, x, co);
  default: return 0.0; /* the reference never asks for order > 3 on its paths */
  }
}

/* y-power scaling of a node's coefficient vectors followed by the Clenshaw
   sums in cb: getff2, src/LIBFILES/getff-new.c:103-156 */
static void node_sums(double res[2], int nf, int nm, int ndy, int ndcb, double y, double cb,
                      const float *fm, const float *fp)
{
  const double y1 = 1.0 / y;
  double yp = 1;
  int mshm = 2;
  switch (nm) {
  case QG0: case dxQG0: case QG1: case dxQG1: case QG3: case dxQG3: case d2xQG3:
    yp = 1.0; mshm = 2; break;
  case QG2: case dxQG2: case d2xQG2: yp = y1; mshm = 3; break;
  case QL4: case dxQL4: yp = y; mshm = 1; break;
  case QL2: case dxQL2: yp = y1 * y1; mshm = 4; break;
  }
  int mshp = 2 - mshm;
  const int mm = abs(mshp);
  double fval[1024 + 4], fvalD[1024 + 4];
  for (int j = 0; j < mm; j++) fval[j] = fvalD[j] = 0.0;
  double facm = y1 * y1 * yp, facp = yp;
  for (int j = 0; j < mm; j++) { facm *= y1; facp *= y; }
  mshm += mm; mshp += mm;
  for (int j = 0; j < nf; j++) {
    fvalD[mm + j] = y1 * mshp * facp * (fp[j]) - y1 * mshm * facm * (fm[j]);
    fval[mm + j] = facm * (fm[j]) + facp * (fp[j]);
    facm *= y1; facp *= y;
    mshm++; mshp++;
  }
  res[1] = chebd(mm + ndcb, nf + mm, cb, fvalD);
  res[0] = ndy ? res[1] : chebd(mm + ndcb, nf + mm, cb, fval);
}

/* accessv, src/LIBFILES/getff-new.c:160-194 */
static double access_y(int flag_hy, int use_y_derivs, int ix, int iy, int nm, int ndy, int ndcb,
                       double cb, double y)
{
  const int nx = G.nfx[ix];
  const double y1 = G.YY[iy];
  double r1[2] = {0., 0.};
  node_sums(r1, nx, nm, ndy, ndcb, y1, cb, FM(nm, ix, iy), FP(nm, ix, iy));
  if (!flag_hy) {
    const int iy2 = iy + 1;
    const double y2 = G.YY[iy2];
    double r2[2] = {0., 0.};
    node_sums(r2, nx, nm, ndy, ndcb, y2, cb, FM(nm, ix, iy2), FP(nm, ix, iy2));
    if (use_y_derivs) return hermite_y(y, y1, y2, y1 - y2, r1[0], r2[0], r1[1], r2[1]);
    return lerp((y2 - y) / (y2 - y1), r1[0], r2[0]);
  }
  return r1[0];
}

/* extractff, scalar path, src/LIBFILES/getff-new.c:213-258 */
static double weight(int nm, int ndy, int ndcb, const inv_t *I)
{
  const int flag_hx = (I->x >= G.XX[G.nstpx - 1]);
  const int flag_hy = (I->y >= G.YY[G.nstpy - 1]);
  const int use_x_derivs = (nm < dxQG0 || nm == dxQG2 || nm == dxQG3);
  const int ix = I->hx.idx, iy = I->hy.idx;
  const int use_y_derivs = !ndy;
  const double f1 = access_y(flag_hy, use_y_derivs, ix, iy, nm, ndy, ndcb, I->cb, I->y);
  if (!flag_hx) {
    const double f2 = access_y(flag_hy, use_y_derivs, ix + 1, iy, nm, ndy, ndcb, I->cb, I->y);
    if (use_x_derivs) {
      const int off = nm < dxQG0 ? dxQG0 : QL4;
      const double g1 = access_y(flag_hy, use_y_derivs, ix, iy, nm + off, ndy, ndcb, I->cb, I->y);
      const double g2 = access_y(flag_hy, use_y_derivs, ix + 1, iy, nm + off, ndy, ndcb, I->cb, I->y);
      return hermite_pre(&I->hx, f1, f2, g1, g2);
    }
    return lerp(I->hx.lA, f1, f2);
  }
  return f1;
}

/* extractff2, scalar path, src/LIBFILES/getff-new.c:295-311:
   F[0] d/dcb, F[1] d/dx, F[2] d/dy, F[3] value */
static void weight4(int nm, int ndcb, const inv_t *I, double F[4])
{
  static const int dxmap[14] = {dxQG0, dxQG1, dxQG2, dxQG3, dxQL4, dxQL2, dxQG0,
                                dxQG1, d2xQG2, d2xQG3, dxQL4, dxQL2, d2xQG2, d2xQG3};
  const int ndcb2 = ndcb + 1 < 5 ? ndcb + 1 : ndcb;
  F[0] = weight(nm, 0, ndcb2, I);
  F[1] = weight(dxmap[nm], 0, ndcb, I);
  F[2] = weight(nm, 1, ndcb, I);
  F[3] = weight(nm, 0, ndcb, I);
}

static void set_grid_pos(inv_t *I)
{
  const int ix1 = bsrch(G.XX, I->x, 0, G.nstpx);
  int ix2 = ix1 + 1;
  if (ix2 >= G.nstpx) ix2 = ix1;
  herm(&I->hx, I->x, G.XX[ix1], G.XX[ix2], ix1);
  const int iy1 = bsrch(G.YY, I->y, 0, G.nstpy);
  int iy2 = iy1 + 1;
  if (iy2 >= G.nstpy) iy2 = iy1;
  herm(&I->hy, I->y, G.YY[iy1], G.YY[iy2], iy1);
}

/* set_invariants, src/LIBFILES/getff-new.c:315-370 */
static void invariants(const double xv[4], const double yv[4], inv_t *I)
{
  const double EPSIN = 1E-7;
  I->xsq = dot4(xv, xv);
  I->xsq = I->xsq < EPSIN ? EPSIN : I->xsq;
  I->x = sqrt(fabs(I->xsq));
  I->ysq = dot4(yv, yv);
  I->ysq = I->ysq < EPSIN ? EPSIN : I->ysq;
  I->y = sqrt(fabs(I->ysq));
  I->xdoty = dot4(xv, yv);
  I->cb = I->xdoty / (I->x * I->y);
  I->cborig = I->cb;
  I->yorig = I->y;
  I->xmysq = (I->xsq + I->ysq) * (1.00000000000001) - 2.0 * I->xdoty;
  I->xmy = sqrt(fabs(I->xmysq));
  I->flag2 = 0;
  const double rx = (I->x > I->xmy ? I->xmy / I->x : I->x / I->xmy);
  const double rxy = (I->x > I->y ? I->y / I->x : I->x / I->y);
  if (rx < rxy && I->xmy < G.YY[G.nstpy - 1] && fabs(I->xmysq) > 1E-28) {
    I->cb = (I->x - I->y * I->cb) / I->xmy;
    I->y = I->xmy;
    I->flag2 = 1;
  }
  set_grid_pos(I);
}

/* The x <-> (x-y) chain rule shared by chnr_dS.c:74-83, chnr_dT.c:240-275 and
   chnr_dV.c:194-216: derivatives of g(x, ca, |x-y|) with respect to
   (x, cb, y); ca = post-swap cb. */
typedef struct { double ca, cd, omc2; } swap_t;
static inline swap_t swap_consts(const inv_t *I)
{
  swap_t s;
  s.ca = I->cb;
  s.cd = (I->yorig - I->x * I->cborig) / I->xmy;
  s.omc2 = 0;
  return s;
}
static inline double swap_dx(const inv_t *I, const swap_t *s, double dx, double dcb, double dy)
{
  return dx + (1.0 - s->ca * s->ca) / I->xmy * dcb + s->ca * dy;
}
static inline double swap_dcb(const inv_t *I, const swap_t *s, double dcb, double dy)
{
  return -(I->ysq * s->cd * dcb + I->x * I->yorig * I->xmy * dy) / I->xmysq;
}
static inline double swap_dy(const inv_t *I, const swap_t *s, double dcb, double dy)
{
  return -(I->cborig + s->ca * s->cd) / I->xmy * dcb + s->cd * dy;
}

/* ---------------------------------------------------------------- chnr_dS */

/* compute_dg_TAYLORX, src/LIBFILES/chnr_dS.c:9-45 */
static int S_taylor(const inv_t *I, double *dg0dy, double *dg0dx, double *dg0dcb)
{
  const int it = bsrch(G.TX[TYY], I->y, 0, G.ny_tay);
  const int iy = bsrch(G.YY, I->y, 0, G.nstpy);
  if (it == G.ny_tay - 1 || iy == G.nstpy - 1) return 1;
  const int it2 = it + 1;
  const double ay = (G.TX[TYY][it2] - I->y) / (G.TX[TYY][it2] - G.TX[TYY][it]);
  const double ax = (G.XX[0] - I->x) / (G.XX[0]);
  double f1 = I->cb * lerp(ay, G.TX[G0dx][it], G.TX[G0dx][it2]);
  double f2 = access_y(0, 1, 0, iy, dxQG0, 0, 0, I->cb, I->y);
  *dg0dx = lerp(ax, f1, f2);
  f1 = lerp(ay, G.TX[G0dy][it], G.TX[G0dy][it2]);
  f2 = access_y(0, 0, 0, iy, QG0, 1, 0, I->cb, I->y);
  *dg0dy = lerp(ax, f1, f2);
  f2 = access_y(0, 1, 0, iy, QG0, 0, 1, I->cb, I->y);
  *dg0dcb = lerp(ax, 0.0, f2);
  return 0;
}

/* chnr_dS, src/LIBFILES/chnr_dS.c:49-95 */
static int build_S(const double xv[4], const double yv[4], const inv_t *I, double dxv[4],
                   double dyv[4])
{
  double dg0dy, dg0dx, dg0dcb;
  if (I->x < G.XX[0]) {
    if (S_taylor(I, &dg0dy, &dg0dx, &dg0dcb)) return 1;
  } else if (I->x > G.XX[G.nstpx - 1]) {
    return 1;
  } else {
    double f[4];
    weight4(QG0, 0, I, f);
    dg0dcb = f[0]; dg0dx = f[1]; dg0dy = f[2];
  }
  if (I->flag2) {
    const swap_t s = swap_consts(I);
    const double ox = dg0dx, ocb = dg0dcb, oy = dg0dy;
    dg0dx = swap_dx(I, &s, ox, ocb, oy);
    dg0dcb = swap_dcb(I, &s, ocb, oy);
    dg0dy = swap_dy(I, &s, ocb, oy);
  }
  for (int b = 0; b < 4; b++) {
    const double yhat = yv[b] / I->yorig;
    const double xhat = xv[b] / I->x;
    const double c2 = (xhat - I->cborig * yhat) / I->yorig;
    const double c4 = (yhat - I->cborig * xhat) / I->x;
    dyv[b] = yhat * dg0dy + c2 * dg0dcb;
    dxv[b] = xhat * dg0dx + c4 * dg0dcb;
  }
  return 0;
}

/* ---------------------------------------------------------------- chnr_dT */

typedef struct {
  double ell1, ell2, ell3, v1, ell4, dv1dx, dv1dy, dv1dcb, dell2dx, dell2dy, dell2dcb;
  double dell1dx, dell1dy, dell1dcb, dell3dx, dell3dy, dell3dcb, dell4dy, dell4dx, dell4dcb;
} tsc_t;

/* TAYLORX_contribution, src/LIBFILES/chnr_dT.c:110-238 */
static int T_taylor(tsc_t *T, const inv_t *I)
{
  const double ysq = I->flag2 ? I->xmysq : I->ysq;
  const int it = bsrch(G.TX[TYY], I->y, 0, G.ny_tay);
  const int iy = bsrch(G.YY, I->y, 0, G.nstpy);
  if (it == G.ny_tay - 1 || iy == G.nstpy - 1) return 1;
  const int it2 = it + 1;
  const double Y = I->y, cb = I->cb;
  const double ay = (G.TX[TYY][it2] - Y) / (G.TX[TYY][it2] - G.TX[TYY][it]);
  const double ax = (G.XX[0] - I->x) / (G.XX[0]);
  const double xb = G.XX[0];
  const double xbsq = xb * xb;
#define TXL(row) lerp(ay, G.TX[row][it], G.TX[row][it2])
  const double ell2a = TXL(Gl2);
  const double ell2b = access_y(0, 1, 0, iy, QL2, 0, 0, cb, Y);
  T->ell2 = lerp(ax, ell2a, ell2b);
  const double dell2adx = TXL(Gl21) * cb;
  const double dell2bdx = access_y(0, 1, 0, iy, dxQL2, 0, 0, cb, Y);
  T->dell2dx = lerp(ax, dell2adx, dell2bdx);
  const double dell2ady = TXL(Gl2dy);
  const double dell2bdy = access_y(0, 0, 0, iy, QL2, 1, 0, cb, Y);
  T->dell2dy = lerp(ax, dell2ady, dell2bdy);
  const double dell2adcb = 0.0;
  const double dell2bdcb = access_y(0, 1, 0, iy, QL2, 0, 1, cb, Y);
  T->dell2dcb = lerp(ax, dell2adcb, dell2bdcb);
  const double v1b = access_y(0, 1, 0, iy, QG1, 0, 0, cb, Y);
  const double dv1bdx = access_y(0, 1, 0, iy, dxQG1, 0, 0, cb, Y);
  const double dv1bdy = access_y(0, 0, 0, iy, QG1, 1, 0, cb, Y);
  const double dv1bdcb = access_y(0, 1, 0, iy, QG1, 0, 1, cb, Y);
  const double ell4b = access_y(0, 1, 0, iy, QL4, 0, 0, cb, Y);
  const double dell4bdx = access_y(0, 1, 0, iy, dxQL4, 0, 0, cb, Y);
  const double dell4bdy = access_y(0, 0, 0, iy, QL4, 1, 0, cb, Y);
  const double dell4bdcb = access_y(0, 1, 0, iy, QL4, 0, 1, cb, Y);
  const double ell3a = TXL(Gl3);
  const double ell3b = ell4b / (2.0 * xbsq * ysq) - Y * cb * ell2b / xb;
  T->ell3 = lerp(ax, ell3a, ell3b);
  const double ell1b = 4.0 / (3.0 * xbsq * xbsq) *
                       (v1b - xbsq * ysq * (cb * cb - 0.25) * ell2b - 1.5 * xbsq * xb * Y * cb * ell3b);
  T->ell1 = ell1b;
  const double dell3ady = TXL(Gl3dy);
  const double dell3bdy =
      (-ell4b / (ysq * Y) + dell4bdy / (2.0 * ysq) - cb * xb * ell2b - Y * xb * cb * dell2bdy) / (xbsq);
  T->dell3dy = lerp(ax, dell3ady, dell3bdy);
  const double dell3adcb = 0.0;
  const double dell3bdcb = (dell4bdcb / (2.0 * xb * ysq) - Y * ell2b - Y * cb * dell2bdcb) / xb;
  T->dell3dcb = lerp(ax, dell3adcb, dell3bdcb);
  const double dell3bdx =
      (-ell4b / (xb * ysq) + dell4bdx / (2.0 * ysq) + Y * cb * ell2b - Y * xb * cb * dell2bdx) / xbsq;
  T->dell3dx = dell3bdx;
  T->dell1dy = 4.0 / (3.0 * xbsq * xbsq) *
               (dv1bdy - 2.0 * xbsq * Y * (cb * cb - 0.25) * ell2b -
                xbsq * ysq * (cb * cb - 0.25) * dell2bdy - 1.5 * xbsq * xb * cb * ell3b -
                1.5 * xbsq * xb * Y * cb * dell3bdy);
  T->dell1dcb = 4.0 / (3.0 * xbsq * xbsq) *
                (dv1bdcb - 2.0 * xbsq * ysq * cb * ell2b - xbsq * ysq * (cb * cb - 0.25) * dell2bdcb -
                 1.5 * xbsq * xb * Y * ell3b - 1.5 * xbsq * xb * Y * cb * dell3bdcb);
  T->dell1dx = -4.0 * ell1b / xb +
               4.0 / (3.0 * xbsq * xbsq) *
                   (dv1bdx - 2.0 * xb * ysq * (cb * cb - 0.25) * ell2b -
                    xbsq * ysq * (cb * cb - 0.25) * dell2bdx - 4.5 * xbsq * Y * cb * ell3b -
                    1.5 * xbsq * xb * Y * cb * dell3bdx);
#undef TXL
  return 0;
}

/* XMYSWAP_T_contrib, src/LIBFILES/chnr_dT.c:240-275 */
static void T_swap(tsc_t *T, const inv_t *I)
{
  const swap_t s = swap_consts(I);
  const double e2x = T->dell2dx, e2cb = T->dell2dcb, e2y = T->dell2dy;
  T->dell2dx = swap_dx(I, &s, e2x, e2cb, e2y);
  T->dell2dcb = swap_dcb(I, &s, e2cb, e2y);
  T->dell2dy = swap_dy(I, &s, e2cb, e2y);
  const double ell3s = -T->ell3, e3x = -T->dell3dx, e3cb = -T->dell3dcb, e3y = -T->dell3dy;
  T->ell3 = ell3s - T->ell2;
  T->dell3dx = swap_dx(I, &s, e3x, e3cb, e3y) - T->dell2dx;
  T->dell3dcb = swap_dcb(I, &s, e3cb, e3y) - T->dell2dcb;
  T->dell3dy = swap_dy(I, &s, e3cb, e3y) - T->dell2dy;
  const double ell1s = T->ell1, e1x = T->dell1dx, e1cb = T->dell1dcb, e1y = T->dell1dy;
  T->ell1 = ell1s - T->ell2 - 2.0 * T->ell3;
  T->dell1dx = swap_dx(I, &s, e1x, e1cb, e1y) - T->dell2dx - 2.0 * T->dell3dx;
  T->dell1dcb = swap_dcb(I, &s, e1cb, e1y) - T->dell2dcb - 2.0 * T->dell3dcb;
  T->dell1dy = swap_dy(I, &s, e1cb, e1y) - T->dell2dy - 2.0 * T->dell3dy;
}

/* chnr_dT, src/LIBFILES/chnr_dT.c:279-388 */
static int build_T(const double xv[4], const double yv[4], const inv_t *I, double dxv[64],
                   double dyv[64])
{
  tsc_t T;
  const double ysq = I->flag2 ? I->xmysq : I->ysq;
  if (I->x < G.XX[0]) {
    if (T_taylor(&T, I)) return 1;
  } else if (I->x > G.XX[G.nstpx - 1]) {
    return 1;
  } else {
    const double X = I->x, Y = I->y, cb = I->cb, xsq = I->xsq;
    double f[4];
    weight4(QL2, 0, I, f);
    T.dell2dx = f[1]; T.dell2dy = f[2]; T.ell2 = f[3]; T.dell2dcb = f[0];
    weight4(QL4, 0, I, f);
    T.dell4dx = f[1]; T.dell4dy = f[2]; T.ell4 = f[3]; T.dell4dcb = f[0];
    weight4(QG1, 0, I, f);
    T.dv1dx = f[1]; T.dv1dy = f[2]; T.v1 = f[3]; T.dv1dcb = f[0];
    T.ell3 = T.ell4 / (2.0 * xsq * ysq) - Y * cb * T.ell2 / X;
    T.ell1 = 4.0 / (3.0 * xsq * xsq) *
             (T.v1 - xsq * ysq * (cb * cb - 0.25) * T.ell2 - 1.5 * xsq * X * Y * cb * T.ell3);
    T.dell3dy = (-T.ell4 / (ysq * Y) + T.dell4dy / (2.0 * ysq) - cb * X * T.ell2 -
                 Y * X * cb * T.dell2dy) / (xsq);
    T.dell3dcb = (T.dell4dcb / (2.0 * X * ysq) - Y * T.ell2 - Y * cb * T.dell2dcb) / X;
    T.dell3dx = (-T.ell4 / (X * ysq) + T.dell4dx / (2.0 * ysq) + Y * cb * T.ell2 -
                 Y * X * cb * T.dell2dx) / xsq;
    T.dell1dy = 4.0 / (3.0 * xsq * xsq) *
                (T.dv1dy - 2.0 * xsq * Y * (cb * cb - 0.25) * T.ell2 -
                 xsq * ysq * (cb * cb - 0.25) * T.dell2dy - 1.5 * xsq * X * cb * T.ell3 -
                 1.5 * xsq * X * Y * cb * T.dell3dy);
    T.dell1dcb = 4.0 / (3.0 * xsq * xsq) *
                 (T.dv1dcb - 2.0 * xsq * ysq * cb * T.ell2 -
                  xsq * ysq * (cb * cb - 0.25) * T.dell2dcb - 1.5 * xsq * X * Y * T.ell3 -
                  1.5 * xsq * X * Y * cb * T.dell3dcb);
    T.dell1dx = -4.0 * T.ell1 / X +
                4.0 / (3.0 * xsq * xsq) *
                    (T.dv1dx - 2.0 * X * ysq * (cb * cb - 0.25) * T.ell2 -
                     xsq * ysq * (cb * cb - 0.25) * T.dell2dx - 4.5 * xsq * Y * cb * T.ell3 -
                     1.5 * xsq * X * Y * cb * T.dell3dx);
  }
  if (I->flag2) T_swap(&T, I);
  for (int b = 0; b < 4; b++) {
    const double c1 = yv[b] / I->yorig;
    const double c3 = xv[b] / I->x;
    const double c2 = (c3 - I->cborig * c1) / I->yorig;
    const double c4 = (c1 - I->cborig * c3) / I->x;
    for (int a = 0; a < 4; a++) {
      const int d_ab = (a == b);
      for (int d = 0; d < 4; d++) {
        const int d_bd = (b == d), d_ad = (a == d);
        const double t1 = d_ab * yv[d] + d_bd * yv[a] - 0.5 * d_ad * yv[b];
        const double t2 = d_ab * xv[d] + d_bd * xv[a] - 0.5 * d_ad * xv[b];
        const double t3 = xv[a] * xv[d] - d_ad * I->xsq / 4;
        const double t4 = yv[a] * yv[d] - d_ad * I->ysq / 4;
        const double t5 = xv[a] * yv[d] + yv[a] * xv[d] - 0.5 * I->xdoty * d_ad;
        const int o = (a * 4 + b) * 4 + d;
        dyv[o] = +t1 * T.ell2 + t2 * T.ell3 + t3 * (c1 * T.dell1dy + c2 * T.dell1dcb) +
                 t4 * (c1 * T.dell2dy + c2 * T.dell2dcb) + t5 * (c1 * T.dell3dy + c2 * T.dell3dcb);
        dxv[o] = +t2 * T.ell1 + t1 * T.ell3 + t3 * (c3 * T.dell1dx + c4 * T.dell1dcb) +
                 t4 * (c3 * T.dell2dx + c4 * T.dell2dcb) + t5 * (c3 * T.dell3dx + c4 * T.dell3dcb);
      }
    }
  }
  return 0;
}

/* ---------------------------------------------------------------- chnr_dV */

typedef struct {
  double g2, dg1dx, dg1dy, dg1dcb, dg2dx, dg2dy, dg2dcb, dg3dx, dg3dy, dg3dcb;
  double ddg2dxdx, ddg2dxdy, ddg2dxdcb, ddg2dydcb, ddg2dcbdcb;
  double ddg3dxdx, ddg3dxdy, ddg3dxdcb, ddg3dydcb, ddg3dcbdcb;
  double ddg1dxdx, ddg1dxdy, ddg1dxdcb, ddg1dydcb, ddg1dcbdcb;
  double ddg1dydy, ddg2dydy;
} vsc_t;

/* taylorx_contrib, src/LIBFILES/chnr_dV.c:18-174 */
static int V_taylor(vsc_t *D, double x, double y, double xsq, int flag2, double cb)
{
  const int it = bsrch(G.TX[TYY], y, 0, G.ny_tay);
  const int iy = bsrch(G.YY, y, 0, G.nstpy);
  if (it == G.ny_tay - 1 || iy == G.nstpy - 1) return 1;
  const int it2 = it + 1;
  const double ay = (G.TX[TYY][it2] - y) / (G.TX[TYY][it2] - G.TX[TYY][it]);
  const double ax = (G.XX[0] - x) / (G.XX[0]);
  const double xb = G.XX[0];
  const double xbsq = xb * xb;
#define TXL(row) lerp(ay, G.TX[row][it], G.TX[row][it2])
  const double g2a = 0.0;
  const double g2b = access_y(0, 1, 0, iy, QG2, 0, 0, cb, y);
  D->g2 = lerp(ax, g2a, g2b);
  const double ddg2adxdcb = TXL(G21);
  const double ddg2bdxdcb = access_y(0, 1, 0, iy, dxQG2, 0, 1, cb, y);
  D->ddg2dxdcb = lerp(ax, ddg2adxdcb, ddg2bdxdcb);
  const double dg2bdx = access_y(0, 1, 0, iy, dxQG2, 0, 0, cb, y);
  D->dg2dx = D->ddg2dxdcb * cb;
  const double dg2bdcb = access_y(0, 1, 0, iy, QG2, 0, 1, cb, y);
  D->dg2dcb = D->ddg2dxdcb * x;
  const double dg2bdy = access_y(0, 0, 0, iy, QG2, 1, 0, cb, y);
  D->dg2dy = lerp(ax, 0.0, dg2bdy);
  const double ddg2adxdy = cb * TXL(G21dy);
  const double ddg2bdxdy = access_y(0, 0, 0, iy, dxQG2, 1, 0, cb, y);
  D->ddg2dxdy = lerp(ax, ddg2adxdy, ddg2bdxdy);
  const double ddg2adxdx = 2.0 * (TXL(G22A) + TXL(G22B) * (0.4 + 0.6 * (2.0 * cb * cb - 1)));
  const double ddg2bdxdx = access_y(0, 1, 0, iy, d2xQG2, 0, 0, cb, y);
  D->ddg2dxdx = lerp(ax, ddg2adxdx, ddg2bdxdx);
  const double ddg2bdcbdcb = access_y(0, 1, 0, iy, QG2, 0, 2, cb, y);
  D->ddg2dcbdcb = ddg2bdcbdcb * xsq / xbsq;
  const double ddg2bdydcb = access_y(0, 0, 0, iy, QG2, 1, 1, cb, y);
  D->ddg2dydcb = lerp(ax, 0.0, ddg2bdydcb);
  const double dg3bdy = access_y(0, 0, 0, iy, QG3, 1, 0, cb, y);
  const double ddg3bdxdy = access_y(0, 0, 0, iy, dxQG3, 1, 0, cb, y);
  const double ddg3bdxdcb = access_y(0, 1, 0, iy, dxQG3, 0, 1, cb, y);
  const double ddg3bdxdx = access_y(0, 1, 0, iy, d2xQG3, 0, 0, cb, y);
  const double ddg3bdcbdcb = access_y(0, 1, 0, iy, QG3, 0, 2, cb, y);
  const double ddg3bdydcb = access_y(0, 0, 0, iy, QG3, 1, 1, cb, y);
  const double dg1bdy = dg3bdy - cb / xb * g2b - (y / xb) * cb * dg2bdy;
  const double ddg1bdxdx = ddg3bdxdx - 2.0 * y / (xbsq * xb) * cb * g2b + y / xbsq * cb * dg2bdx +
                           y / xbsq * cb * dg2bdx - y / xb * cb * ddg2bdxdx;
  const double ddg1bdxdy = ddg3bdxdy + cb / xbsq * g2b + y * cb / xbsq * dg2bdy - cb / xb * dg2bdx -
                           y / xb * cb * ddg2bdxdy;
  const double ddg1bdxdcb = ddg3bdxdcb + y / xbsq * g2b + y / xbsq * cb * dg2bdcb - y / xb * dg2bdx -
                            y / xb * cb * ddg2bdxdcb;
  const double ddg1bdydcb = ddg3bdydcb - g2b / xb - cb / xb * dg2bdcb - y / xb * dg2bdy -
                            y / xb * cb * ddg2bdydcb;
  const double ddg1bdcbdcb = ddg3bdcbdcb - 2.0 * y / xb * dg2bdcb - y / xb * cb * ddg2bdcbdcb;
  const double dg1ady = TXL(G3Ady) - TXL(G3Bdy);
  const double ddg1adxdy = cb * (TXL(G31Ady) - (2 / 3.) * TXL(G31Bdy) - TXL(G22A) - y * TXL(G22Ady));
  const double ddg1adxdcb = TXL(G31A) - (2 / 3.) * TXL(G31B) - y * TXL(G22A);
  const double ddg1adxdx = ddg1bdxdx;
  D->ddg1dxdcb = lerp(ax, ddg1adxdcb, ddg1bdxdcb);
  D->dg1dx = D->ddg1dxdcb * cb;
  D->dg1dcb = D->ddg1dxdcb * x;
  D->dg1dy = lerp(ax, dg1ady, dg1bdy);
  D->ddg1dxdy = lerp(ax, ddg1adxdy, ddg1bdxdy);
  D->ddg1dxdx = lerp(ax, ddg1adxdx, ddg1bdxdx);
  D->ddg1dcbdcb = ddg1bdcbdcb * xsq / xbsq;
  D->ddg1dydcb = lerp(ax, 0.0, ddg1bdydcb);
  if (flag2) {
    const double ya = G.YY[iy];
    const double yb = G.YY[iy + 1];
    const double ddg2adydy = 0.0;
    const double dg2bdy_ya = access_y(0, 0, 0, iy, QG2, 1, 0, cb, ya);
    const double dg2bdy_yb = access_y(0, 0, 0, iy, QG2, 1, 0, cb, yb);
    const double ddg2bdydy = (dg2bdy_yb - dg2bdy_ya) / G.ystp;
    D->ddg2dydy = ax * ddg2adydy + (1.0 - ax) * ddg2bdydy;
    const double ddg1adydy = (G.TX[G3Ady][it2] - G.TX[G3Bdy][it2] - (G.TX[G3Ady][it] - G.TX[G3Bdy][it])) /
                             (G.TX[TYY][it2] - G.TX[TYY][it]);
    const double dg3bdy_ya = access_y(0, 0, 0, iy, QG3, 1, 0, cb, ya);
    const double dg3bdy_yb = access_y(0, 0, 0, iy, QG3, 1, 0, cb, yb);
    const double ddg3bdydy = (dg3bdy_yb - dg3bdy_ya) / G.ystp;
    const double ddg1bdydy = ddg3bdydy - (y * ddg2bdydy + 2.0 * dg2bdy) * cb / x;
    D->ddg1dydy = ax * ddg1adydy + (1.0 - ax) * ddg1bdydy;
  }
#undef TXL
  return 0;
}

/* XMYSWAP_V_contrib with v_flip2, src/LIBFILES/chnr_dV.c:176-274.
   x, xmy, y(=|y| original), xsq, xmysq, ysq, ca (post-swap cb), cborig */
static void V_swap(vsc_t *D, double x, double xmy, double y, double xsq, double xmysq, double ysq,
                   double ca, double cborig)
{
  vsc_t F = *D;
  F.g2 = -D->g2; F.dg2dx = -D->dg2dx; F.dg2dy = -D->dg2dy; F.dg2dcb = -D->dg2dcb;
  F.ddg2dxdx = -D->ddg2dxdx; F.ddg2dxdy = -D->ddg2dxdy; F.ddg2dydy = -D->ddg2dydy;
  F.ddg2dxdcb = -D->ddg2dxdcb; F.ddg2dydcb = -D->ddg2dydcb; F.ddg2dcbdcb = -D->ddg2dcbdcb;
  const double cd = (y - x * cborig) / xmy;

  D->g2 = F.g2;
  D->dg2dx = F.dg2dx + (1.0 - ca * ca) / xmy * F.dg2dcb + ca * F.dg2dy;
  D->dg2dcb = -(ysq * cd * F.dg2dcb + x * y * xmy * F.dg2dy) / xmysq;
  D->dg2dy = -(cborig + ca * cd) / xmy * F.dg2dcb + cd * F.dg2dy;

  D->dg1dx = F.dg1dx + (1.0 - ca * ca) / xmy * F.dg1dcb + ca * F.dg1dy - D->dg2dx;
  D->dg1dcb = -(ysq * cd * F.dg1dcb + x * y * xmy * F.dg1dy) / xmysq - D->dg2dcb;
  D->dg1dy = -(cborig + ca * cd) / xmy * F.dg1dcb + cd * F.dg1dy - D->dg2dy;

  /* second derivatives of g2, then of g1 (which subtract g2's) */
#define DXDX(g)                                                                              \
  ((F.ddg##g##dxdx + (1.0 - ca * ca) / xmy * F.ddg##g##dxdcb + ca * F.ddg##g##dxdy) -          \
   3.0 * ca * (1.0 - ca * ca) / xmysq * F.dg##g##dcb +                                       \
   (1.0 - ca * ca) / xmy * (F.ddg##g##dxdcb + (1.0 - ca * ca) / xmy * F.ddg##g##dcbdcb + ca * F.ddg##g##dydcb) + \
   (1.0 - ca * ca) / xmy * F.dg##g##dy +                                                     \
   ca * (F.ddg##g##dxdy + (1.0 - ca * ca) / xmy * F.ddg##g##dydcb + ca * F.ddg##g##dydy))
#define DXDCB(g)                                                                             \
  (ysq / (xmysq * xmy) * (cborig + 3.0 * ca * cd) * F.dg##g##dcb -                            \
   ysq / xmysq * cd * (F.ddg##g##dxdcb + (1.0 - ca * ca) / xmy * F.ddg##g##dcbdcb + ca * F.ddg##g##dydcb) + \
   y / xmysq * (x * ca - xmy) * F.dg##g##dy -                                                \
   x * y / xmy * (F.ddg##g##dxdy + (1.0 - ca * ca) / xmy * F.ddg##g##dydcb + ca * F.ddg##g##dydy))
#define DXDY(g)                                                                              \
  ((-(cborig + ca * cd) / xmy * F.ddg##g##dxdcb + cd * F.ddg##g##dxdy) +                      \
   (2.0 * ca * cborig + cd * (3.0 * ca * ca - 1.0)) / xmysq * F.dg##g##dcb +                  \
   (1.0 - ca * ca) / xmy * (-(cborig + ca * cd) / xmy * F.ddg##g##dcbdcb + cd * F.ddg##g##dydcb) - \
   (cborig + ca * cd) / xmy * F.dg##g##dy +                                                  \
   ca * (-(cborig + ca * cd) / xmy * F.ddg##g##dydcb + cd * F.ddg##g##dydy))
#define DYDCB(g)                                                                             \
  (y / (xmysq * xmy) * ((3.0 * cd * cd - 1.0) * y - 2 * xmy * cd) * F.dg##g##dcb -            \
   ysq / (xmysq)*cd * (-(cborig + ca * cd) / xmy * F.ddg##g##dcbdcb + cd * F.ddg##g##dydcb) +  \
   x / xmysq * (y * cd - xmy) * F.dg##g##dy -                                                \
   x * y / xmy * (-(cborig + ca * cd) / xmy * F.ddg##g##dydcb + cd * F.ddg##g##dydy))
#define DCBDCB(g)                                                                            \
  (x * ysq / (xmysq * xmysq) * (xmy - 3.0 * y * cd) * F.dg##g##dcb -                          \
   ysq / (xmysq)*cd * (-(ysq * cd * F.ddg##g##dcbdcb + x * y * xmy * F.ddg##g##dydcb) / xmysq) - \
   xsq * ysq / (xmysq * xmy) * F.dg##g##dy -                                                 \
   x * y / xmy * (-(ysq * cd * F.ddg##g##dydcb + x * y * xmy * F.ddg##g##dydy) / xmysq))

  D->ddg2dxdx = DXDX(2);
  D->ddg2dxdcb = DXDCB(2);
  D->ddg2dxdy = DXDY(2);
  D->ddg2dydcb = DYDCB(2);
  D->ddg2dcbdcb = DCBDCB(2);
  D->ddg1dxdx = DXDX(1) - D->ddg2dxdx;
  D->ddg1dxdcb = DXDCB(1) - D->ddg2dxdcb;
  D->ddg1dxdy = DXDY(1) - D->ddg2dxdy;
  D->ddg1dydcb = DYDCB(1) - D->ddg2dydcb;
  D->ddg1dcbdcb = DCBDCB(1) - D->ddg2dcbdcb;
#undef DXDX
#undef DXDCB
#undef DXDY
#undef DYDCB
#undef DCBDCB
}

/* get_dv, src/LIBFILES/chnr_dV.c:277-359 */
static void V_assemble(double x, const double xv[4], double y, const double yv[4], double cb,
                       const vsc_t *D, double dv[64])
{
  double xhat[4], yhat[4], c2v[4], c4v[4];
  double D1[4], D2[4], D3[4], D4[4], D5[4], D6[4], D7[4], D8[4];
  for (int m = 0; m < 4; m++) { xhat[m] = xv[m] / x; yhat[m] = yv[m] / y; }
  for (int m = 0; m < 4; m++) {
    c2v[m] = (xhat[m] - cb * yhat[m]) / y;
    c4v[m] = (yhat[m] - cb * xhat[m]) / x;
    D1[m] = xv[m] * D->ddg1dxdx + yv[m] * D->ddg2dxdx;
    D2[m] = xv[m] * D->ddg1dxdy + yv[m] * D->ddg2dxdy;
    D3[m] = xv[m] * D->ddg1dxdcb + yv[m] * D->ddg2dxdcb;
    D4[m] = xv[m] * D->ddg1dydcb + yv[m] * D->ddg2dydcb;
    D5[m] = xv[m] * D->ddg1dxdcb + yv[m] * D->ddg2dxdcb;
    D6[m] = xv[m] * D->ddg1dcbdcb + yv[m] * D->ddg2dcbdcb;
    D7[m] = (xv[m] * D->dg1dx + yv[m] * D->dg2dx) / x;
    D8[m] = (xv[m] * D->dg1dcb + yv[m] * D->dg2dcb) / x;
  }
  for (int a = 0; a < 4; a++) {
    const double astuff = (D->dg1dx + D->dg2dx) * xhat[a] + (D->dg1dcb + D->dg2dcb) * c4v[a];
    for (int b = 0; b < 4; b++) {
      const double bstuff = (D->dg1dx * xhat[b] + D->dg1dy * yhat[b] +
                             D->dg1dcb * (xhat[b] / y + yhat[b] / x - cb * (xhat[b] / x + yhat[b] / y)));
      const double c2c4 = c2v[b] + c4v[b];
      const int d_ab = (a == b);
      const double xaxb = xhat[a] * xhat[b], yayb = yhat[a] * yhat[b];
      const double xayb = xhat[a] * yhat[b], yaxb = yhat[a] * xhat[b];
      const double c1 = ((cb * (3.0 * xaxb - d_ab) - xayb - yaxb) / x + (d_ab + xayb * cb - xaxb - yayb) / y);
      for (int d = 0; d < 4; d++) {
        const int d_bd = (b == d), d_ad = (a == d);
        double f = d_bd * astuff;
        f += d_ad * bstuff;
        f += D1[d] * xaxb + D2[d] * xayb;
        f += (D3[d] * xhat[b] + D4[d] * yhat[b]) * c4v[a];
        f += (D5[d] * xhat[a] + D6[d] * c4v[a]) * c2c4;
        f += D7[d] * (d_ab - xaxb);
        dv[(a * 4 + b) * 4 + d] = f + D8[d] * c1;
      }
    }
  }
}

/* chnr_dV, src/LIBFILES/chnr_dV.c:361-479 */
static int build_V(const double xv[4], const double yv[4], const inv_t *I, double dv[64])
{
  vsc_t D;
  memset(&D, 0, sizeof(D));
  if (I->x < G.XX[0]) {
    if (V_taylor(&D, I->x, I->y, I->xsq, I->flag2, I->cb)) return 1;
  } else if (I->x > G.XX[G.nstpx - 1]) {
    return 1;
  } else {
    const double X = I->x, Y = I->y, cb = I->cb, xsq = I->xsq;
    D.dg3dy = weight(QG3, 1, 0, I);
    double f[4];
    weight4(QG2, 0, I, f);
    D.g2 = f[3]; D.dg2dy = f[2];
    weight4(dxQG2, 0, I, f);
    D.ddg2dxdx = f[1]; D.dg2dx = f[3]; D.ddg2dxdy = f[2]; D.ddg2dxdcb = f[0];
    weight4(dxQG3, 0, I, f);
    D.ddg3dxdx = f[1]; D.dg3dx = f[3]; D.ddg3dxdy = f[2]; D.ddg3dxdcb = f[0];
    weight4(QG2, 1, I, f);
    D.dg2dcb = f[3]; D.ddg2dydcb = f[2]; D.ddg2dcbdcb = f[0];
    weight4(QG3, 1, I, f);
    D.dg3dcb = f[3]; D.ddg3dydcb = f[2]; D.ddg3dcbdcb = f[0];
    D.dg1dx = D.dg3dx + Y / xsq * cb * D.g2 - Y / X * cb * D.dg2dx;
    D.dg1dy = D.dg3dy - cb / X * D.g2 - (Y / X) * cb * D.dg2dy;
    D.dg1dcb = D.dg3dcb - Y / X * D.g2 - Y / X * cb * D.dg2dcb;
    D.ddg1dxdx = D.ddg3dxdx - 2.0 * Y / (xsq * X) * cb * D.g2 + Y / xsq * cb * D.dg2dx +
                 Y / xsq * cb * D.dg2dx - Y / X * cb * D.ddg2dxdx;
    D.ddg1dxdy = D.ddg3dxdy + cb / xsq * D.g2 + Y * cb / xsq * D.dg2dy - cb / X * D.dg2dx -
                 Y / X * cb * D.ddg2dxdy;
    D.ddg1dxdcb = D.ddg3dxdcb + Y / xsq * D.g2 + Y / xsq * cb * D.dg2dcb - Y / X * D.dg2dx -
                  Y / X * cb * D.ddg2dxdcb;
    D.ddg1dydcb = D.ddg3dydcb - D.g2 / X - cb / X * D.dg2dcb - Y / X * D.dg2dy -
                  Y / X * cb * D.ddg2dydcb;
    D.ddg1dcbdcb = D.ddg3dcbdcb - 2.0 * Y / X * D.dg2dcb - Y / X * cb * D.ddg2dcbdcb;
    if (I->flag2) {
      const int iy1 = bsrch(G.YY, Y, 0, G.nstpy);
      if (iy1 == G.nstpy - 1) return 1;
      inv_t I1 = *I, I2 = *I;
      I1.y = G.YY[iy1];
      I2.y = G.YY[iy1 + 1];
      double q1 = weight(QG2, 1, 0, &I1), q2 = weight(QG2, 1, 0, &I2);
      D.ddg2dydy = (q2 - q1) / G.ystp;
      q1 = weight(QG3, 1, 0, &I1);
      q2 = weight(QG3, 1, 0, &I2);
      const double ddg3dydy = (q2 - q1) / G.ystp;
      D.ddg1dydy = ddg3dydy - (Y * D.ddg2dydy + 2.0 * D.dg2dy) * cb / X;
    }
  }
  if (I->flag2) V_swap(&D, I->x, I->xmy, I->yorig, I->xsq, I->xmysq, I->ysq, I->cb, I->cborig);
  V_assemble(I->x, xv, I->yorig, yv, I->cborig, &D, dv);
  return 0;
}

/* ------------------------------------------------------- kernel assembly */

/* the fixed STV(200) -> 384 linear maps, CONSTRUCT_FULL_KERNEL
   (src/LIBFILES/QED_kernel.c:16-423) and CONSTRUCT_KERNEL_FULL_EQZERO
   (src/LIBFILES/QED_kernel_xy0.c:8-399) */
static void apply_map(const unsigned short *row, const unsigned char *col, const signed char *q4,
                      const double *stv, double *out)
{
  for (int r = 0; r < 384; r++) {
    double s = 0.0;
    for (int k = row[r]; k < row[r + 1]; k++) s += (q4[k] * 0.25) * stv[col[k]];
    out[r] = s;
  }
}

/* kernelQED + init_STV, src/LIBFILES/QED_kernel.c:427-538 (portable path) */
static int kernel_generic(const double xv[4], const double yv[4], double *out)
{
  inv_t I;
  invariants(xv, yv, &I);
  double stv[200];
  memset(stv, 0, sizeof(stv));
  if (build_S(xv, yv, &I, stv + 0, stv + 4) || build_T(xv, yv, &I, stv + 8, stv + 72) ||
      build_V(xv, yv, &I, stv + 136))
    return 1;
  apply_map(KQ_MAP_GEN_ROW, KQ_MAP_GEN_COL, KQ_MAP_GEN_Q4, stv, out);
  return 0;
}

static const double dlta[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};

/* Tabd_xeq0, src/LIBFILES/Tabd.c:22-114; tI -> V, tII -> Tx, tIII -> Ty */
static int tabd_x0(const double yv[4], double *tI, double *tII, double *tIII)
{
  const double ysq = dot4(yv, yv);
  const double y = sqrt(fabs(ysq));
  const int it = bsrch(G.TX[TYY], y, 0, G.ny_tay);
  if (it == G.ny_tay - 1) return 1;
  const int it2 = it + 1;
  const double ay = (G.TX[TYY][it2] - y) / (G.TX[TYY][it2] - G.TX[TYY][it]);
#define TXL(row) lerp(ay, G.TX[row][it], G.TX[row][it2])
  const double fx = 0.5 * TXL(G0dx);
  const double fy = 0.5 * TXL(G0dy);
  const double yhat[4] = {yv[0] / y, yv[1] / y, yv[2] / y, yv[3] / y};
  double dg0dy[4], dg0dx[4];
  for (int m = 0; m < 4; m++) { dg0dy[m] = yhat[m] * fy / 2; dg0dx[m] = yhat[m] * fx / 2; }
  const double ell2 = TXL(Gl2);
  const double dell2adx = TXL(Gl21);
  const double dell2ady = TXL(Gl2dy);
  const double ell3a = TXL(Gl3);
  const double dg2dx = TXL(G21);
  const double ddg2dxdy = TXL(G21dy);
  const double dg1dx = (TXL(G31A) - (2. / 3) * (TXL(G31B)) - y * (TXL(G22A)));
  const double dg1dy = (TXL(G3Ady) - TXL(G3Bdy));
  const double phi1 = (TXL(G22A) - TXL(G22B) / 5.);
  const double phi2 = (TXL(G22B)) * 1.2;
#undef TXL
  const double ysq_4 = ysq / 4.;
  const double E = (ell3a + ell2), D2 = (dell2adx + dell2ady), D1 = (dg1dy + dg1dx),
               D12 = (dg1dx + dg2dx), D3 = (y * ddg2dxdy - dg2dx);
  double yvE[4], yvell3a[4], yhatD1[4], yhatD2[4], yhatD3[4], yhatdg2dx[4];
  for (int m = 0; m < 4; m++) {
    yvE[m] = yv[m] * E; yvell3a[m] = yv[m] * ell3a; yhatD1[m] = yhat[m] * D1;
    yhatD2[m] = yhat[m] * D2; yhatD3[m] = yhat[m] * D3; yhatdg2dx[m] = yhat[m] * dg2dx;
  }
  int o = 0;
  for (int a = 0; a < 4; a++) {
    const double yalf2dx = yhat[a] * (dell2adx);
    const double tIIsum = dg0dx[a] - 0.5 * yvell3a[a] - ysq_4 * yalf2dx;
    const double yD12 = yhat[a] * D12;
    for (int b = 0; b < 4; b++) {
      const double dgSUM = (dg0dx[b] + dg0dy[b]);
      const double tIsum = 2 * (dlta[a][b] * phi1 + yhat[a] * yhat[b] * phi2);
      const double tIIIsum = dgSUM - 0.5 * yvE[b] - ysq_4 * yhatD2[b];
      for (int d = 0; d < 4; d++, o++) {
        tIII[o] = (yv[a] * yv[d] * yhatD2[b] + dlta[a][b] * yvE[d] + dlta[b][d] * yvE[a] +
                   dlta[a][d] * tIIIsum);
        tII[o] = (yv[b] * yv[d] * yalf2dx + dlta[b][d] * (tIIsum) +
                  (dlta[b][a] * yvell3a[d] + dlta[a][d] * yvell3a[b]));
        tI[o] = (dlta[b][d] * yD12 + yhatdg2dx[d] * dlta[a][b] + yhatD3[b] * yhat[a] * yhat[d] +
                 yhatD1[b] * dlta[a][d] + yv[d] * tIsum);
      }
    }
  }
  return 0;
}

/* Tabd_yeq0, src/LIBFILES/Tabd.c:116-217 (the loop form; the reference's
   unrolled form at :218-313 computes the same expressions) */
static int tabd_y0(const double xv[4], double *tI, double *tII, double *tIII)
{
  const double xsq = dot4(xv, xv);
  const double x = sqrt(fabs(xsq));
  int ix = bsrch(G.XX, x, 0, G.nstpx);
  if (x > G.XX[G.nstpx - 1]) return 1;
  /* |x| exactly on the last node: the reference reads XX[nstpx] here
     (one past its grid); interpolate from the last interval instead */
  if (ix == G.nstpx - 1) ix = G.nstpx - 2;
  const int ix2 = ix + 1;
  const double ax = (G.XX[ix2] - x) / (G.XX[ix2] - G.XX[ix]);
  const double xa = G.XX[ix], xb = G.XX[ix2];
  const double *const *TY = (const double *const *)G.TY;
  const double fx = 0.5 * lerp(ax, TY[alpha0dx_0p][ix], TY[alpha0dx_0p][ix2]);
  const double fy = (lerp(ax, TY[alpha0_1p][ix], TY[alpha0_1p][ix2]));
  const double xhat[4] = {xv[0] / x, xv[1] / x, xv[2] / x, xv[3] / x};
  double dg0dy[4], dg0dx[4];
  for (int m = 0; m < 4; m++) { dg0dy[m] = xhat[m] * fy / 2; dg0dx[m] = xhat[m] * fx / 2; }
  const double xa2 = xa * xa, xa3 = xa2 * xa, xa4 = xa3 * xa;
  const double xb2 = xb * xb, xb3 = xb2 * xb, xb4 = xb3 * xb;
  const double ell1 = 4 * (lerp(ax, TY[alpha1_0p][ix] / (xa4), TY[alpha1_0p][ix2] / (xb4))) / 3.;
  const double ell3 = lerp(ax, TY[beta4_1p][ix] / (xa2), TY[beta4_1p][ix2] / (xb2));
  const double dell1dx = 4 * lerp(ax, (TY[alpha1dx_0p][ix] - 4. * TY[alpha1_0p][ix] / xa) / xa4,
                                  (TY[alpha1dx_0p][ix2] - 4. * TY[alpha1_0p][ix2] / xb) / xb4) / 3.;
  const double dell1dycb = 2 * lerp(ax, (4. * TY[alpha1_1p][ix] / (3 * xa) - TY[beta4_1p][ix]) / xa3,
                                    (4. * TY[alpha1_1p][ix2] / (3 * xb) - TY[beta4_1p][ix2]) / xb3);
  const double dg1dx = lerp(ax, TY[alpha3dx_0p][ix], TY[alpha3dx_0p][ix2]);
  const double ddg1dxdx = lerp(ax, TY[alpha3dxdx_0p][ix], TY[alpha3dxdx_0p][ix2]);
  const double dg2dx = 2 * lerp(ax, TY[beta2dx_1p][ix], TY[beta2dx_1p][ix2]);
  const double dg1dycb = 2 * lerp(ax, TY[alpha3_1p][ix] - TY[beta2_1p][ix] / xa,
                                  TY[alpha3_1p][ix2] - TY[beta2_1p][ix2] / xb);
  const double ddg1dxdycb = 2 * lerp(ax, TY[beta2_1p][ix] / (xa2) - TY[beta2dx_1p][ix] / xa + TY[alpha3dx_1p][ix],
                                     TY[beta2_1p][ix2] / (xb2) - TY[beta2dx_1p][ix2] / xb + TY[alpha3dx_1p][ix2]);
  const double xsq_4 = xsq / 4., E = ell1 + ell3, D1 = dell1dx + dell1dycb,
               D2 = (ddg1dxdx + ddg1dxdycb), D3 = (dg1dycb - dg2dx), D4 = (dg1dx + dg1dycb);
  double xvE[4], xvell1[4];
  for (int m = 0; m < 4; m++) { xvE[m] = xv[m] * E; xvell1[m] = xv[m] * ell1; }
  int o = 0;
  for (int a = 0; a < 4; a++) {
    const double xhd1dx = xhat[a] * (dell1dx);
    const double tIIsum = (dg0dx[a] - 0.5 * xvell1[a]);
    for (int b = 0; b < 4; b++) {
      const double Dg0SUM = (dg0dx[b] + dg0dy[b] - 0.5 * xvE[b]);
      for (int d = 0; d < 4; d++, o++) {
        const double xad = (xv[a] * xv[d] - xsq_4 * dlta[a][d]);
        tIII[o] = ((xad * xhat[b] * D1 + dlta[a][b] * xvE[d] + dlta[b][d] * xvE[a] + Dg0SUM * dlta[a][d]));
        tII[o] = ((xv[b] * xv[d] - xsq_4 * dlta[b][d]) * xhd1dx + dlta[b][a] * xvell1[d] +
                  dlta[a][d] * xvell1[b] + dlta[b][d] * (tIIsum));
        tI[o] = ((dlta[a][d] * xhat[b] + dlta[b][d] * xhat[a] + dlta[a][b] * xhat[d] -
                  xhat[a] * xhat[b] * xhat[d]) * D4 +
                 xhat[a] * (xhat[b] * xv[d] * D2 - dlta[b][d] * D3));
      }
    }
  }
  return 0;
}

/* kernelQED_xoryeq0, src/LIBFILES/QED_kernel_xy0.c:403-427 */
static int kernel_axis(const double qv[4], int xzero, double *out)
{
  double stv[200];
  memset(stv, 0, sizeof(stv));
  const int bad = xzero ? tabd_x0(qv, stv + 136, stv + 8, stv + 72)
                        : tabd_y0(qv, stv + 136, stv + 8, stv + 72);
  if (bad) return 1;
  apply_map(KQ_MAP_ZERO_ROW, KQ_MAP_ZERO_COL, KQ_MAP_ZERO_Q4, stv, out);
  return 0;
}

/* is_zero / x_is_y, src/LIBFILES/kernels.c:13-26 */
static inline int is_zero(const double *v) { return (v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3]) < 1E-28; }

/* QED_kernel_L0, src/LIBFILES/kernels.c:81-115; returns the branch code */
static int L0(const double xv[4], const double yv[4], double *out)
{
  memset(out, 0, 384 * sizeof(double));
  /* non-finite input: zero kernel, reported as out of grid (the reference's
     grid search would run off its tables) */
  if (!isfinite(fabs(xv[0]) + fabs(xv[1]) + fabs(xv[2]) + fabs(xv[3]) + fabs(yv[0]) +
                fabs(yv[1]) + fabs(yv[2]) + fabs(yv[3])))
    return 16 | 4;
  const int x0 = is_zero(xv), y0 = is_zero(yv);
  if (x0 && y0) return 0;
  if (x0) return kernel_axis(yv, 1, out) ? 16 | 1 : 1;
  if (y0) return kernel_axis(xv, 0, out) ? 16 | 2 : 2;
  const double d[4] = {xv[0] - yv[0], xv[1] - yv[1], xv[2] - yv[2], xv[3] - yv[3]};
  if (is_zero(d)) {
    if (kernel_axis(xv, 0, out)) { memset(out, 0, 384 * sizeof(double)); return 16 | 3; }
    /* kernel_mulam_minus, kernels.c:37-48: L -> -L with mu <-> lambda */
    double t[384];
    memcpy(t, out, sizeof(t));
    for (int i = 0; i < 384; i++) {
      const int rs = i / 64, mu = (i / 16) & 3, nu = (i / 4) & 3, la = i & 3;
      out[i] = -t[rs * 64 + la * 16 + nu * 4 + mu];
    }
    return 3;
  }
  if (kernel_generic(xv, yv, out)) { memset(out, 0, 384 * sizeof(double)); return 16 | 4; }
  return 4;
}

/* atomic_kernel_Saxpy, kernels.c:50-78 */
static inline void axpy(double *k, double s, const double *t)
{
  for (int i = 0; i < 384; i++) k[i] += t[i] * s;
}

/* QED_kernel_L1/L2/L3, src/LIBFILES/kernels.c:117-177 */
static void Lvar(int variant, const double *xv, const double *yv, double *out)
{
  static const double zero[4] = {0, 0, 0, 0};
  double t[384];
  L0(xv, yv, out);
  switch (variant) {
  case 1:
    L0(xv, xv, t); axpy(out, -0.5, t);
    L0(yv, yv, t); axpy(out, -0.5, t);
    break;
  case 2:
    L0(zero, yv, t); axpy(out, -1, t);
    L0(xv, zero, t); axpy(out, -1, t);
    break;
  case 3:
    L0(xv, xv, t); axpy(out, -1, t);
    L0(zero, xv, t); axpy(out, +1, t);
    L0(zero, yv, t); axpy(out, -1, t);
    break;
  default: break;
  }
}

int oracle_kernel(int variant, long n, const double *x, const double *y, double *out, int nthreads)
{
  if (!G_ready || variant < 0 || variant > 3) return 1;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
#endif
  for (long i = 0; i < n; i++) Lvar(variant, x + 4 * i, y + 4 * i, out + 384 * i);
  return 0;
}

/* one L0 evaluation for the composite-kernel restatements
   (kqed_composite_oracle.c) */
int oracle_L0_one(const double xv[4], const double yv[4], double *out)
{
  if (!G_ready) return 1;
  L0(xv, yv, out);
  return 0;
}

int oracle_contract(int variant, long n, const double *x, const double *y, const double *pi,
                    double *dots, int nthreads)
{
  if (!G_ready || variant < 0 || variant > 3) return 1;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
#endif
  for (long i = 0; i < n; i++) {
    double k[384];
    Lvar(variant, x + 4 * i, y + 4 * i, k);
    const double *p = pi + 384 * i;
    double s = 0.0;
    for (int c = 0; c < 384; c++) s += k[c] * p[c];
    dots[i] = s;
  }
  return 0;
}

/* the 200 STV components of generic pairs (zero vector for other branches) */
int oracle_stv(long n, const double *x, const double *y, double *out)
{
  if (!G_ready) return 1;
  for (long i = 0; i < n; i++) {
    double *o = out + 200 * i;
    memset(o, 0, 200 * sizeof(double));
    inv_t I;
    const double *xv = x + 4 * i, *yv = y + 4 * i;
    if (is_zero(xv) || is_zero(yv)) continue;
    invariants(xv, yv, &I);
    if (build_S(xv, yv, &I, o + 0, o + 4) || build_T(xv, yv, &I, o + 8, o + 72) ||
        build_V(xv, yv, &I, o + 136))
      memset(o, 0, 200 * sizeof(double));
  }
  return 0;
}

int oracle_branch(long n, const double *x, const double *y, int *code)
{
  if (!G_ready) return 1;
  for (long i = 0; i < n; i++) {
    double k[384];
    int c = L0(x + 4 * i, y + 4 * i, k);
    if ((c & 15) == 4) {
      inv_t I;
      invariants(x + 4 * i, y + 4 * i, &I);
      if (I.x < G.XX[0]) c = (c & 16) | 5;
      if (I.flag2) c |= 8;
    }
    code[i] = c;
  }
  return 0;
}

int oracle_weights(long n, const double *X, const double *Y, const double *CB, double *out,
                   int nthreads)
{
  if (!G_ready) return 1;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
#endif
  for (long i = 0; i < n; i++) {
    inv_t I;
    memset(&I, 0, sizeof(I));
    I.x = X[i]; I.y = Y[i]; I.cb = CB[i];
    I.xsq = X[i] * X[i]; I.ysq = Y[i] * Y[i];
    set_grid_pos(&I);
    double *o = out + 37 * i;
    weight4(QG0, 0, &I, o + 0);
    weight4(QL2, 0, &I, o + 4);
    weight4(QL4, 0, &I, o + 8);
    weight4(QG1, 0, &I, o + 12);
    weight4(QG2, 0, &I, o + 16);
    weight4(dxQG2, 0, &I, o + 20);
    weight4(dxQG3, 0, &I, o + 24);
    weight4(QG2, 1, &I, o + 28);
    weight4(QG3, 1, &I, o + 32);
    o[36] = weight(QG3, 1, 0, &I);
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* Synthetic Pi of the generated-Pi lattice sums (a benchmark input, not part
   of the reference): Philox-4x32-10 (Salmon et al., SC'11) keyed by the
   seed, counter (n0 + n, k0 + k, q, stream); component c takes word (c >> 5) & 3 of
   call q = (c & 31) + 32 (c >> 7); value (b0+b1+b2+b3 - 510) sqrt(3)/256 of
   that word's bytes, times exp(-(|y| + |x - y|) / 2). */
static void philox10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
  for (int r = 0; r < 10; r++) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = (uint32_t)p1;
    c[2] = n2;
    c[3] = (uint32_t)p0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

int oracle_pi_synth(long nx, const double *x, long ny, const double *y, uint64_t seed,
                    uint32_t stream, long k0, long n0, double *pi)
{
  for (long k = 0; k < nx; k++)
    for (long n = 0; n < ny; n++) {
      const double *xv = x + 4 * k, *yv = y + 4 * n;
      const double d0 = xv[0] - yv[0], d1 = xv[1] - yv[1], d2 = xv[2] - yv[2], d3 = xv[3] - yv[3];
      const double nyv = sqrt(yv[0] * yv[0] + yv[1] * yv[1] + yv[2] * yv[2] + yv[3] * yv[3]);
      const double nd = sqrt(d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3);
      const double env = exp(-0.5 * (nyv + nd));
      double *out = pi + (k * ny + n) * 384;
      for (int q = 0; q < 96; q++) {
        uint32_t c[4] = {(uint32_t)(n0 + n), (uint32_t)(k0 + k), (uint32_t)q, stream};
        philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        for (int w = 0; w < 4; w++) {
          const uint32_t v = c[w];
          const int s = (int)(v & 0xffu) + (int)((v >> 8) & 0xffu) + (int)((v >> 16) & 0xffu) +
                        (int)(v >> 24);
          out[(4 * (q >> 5) + w) * 32 + (q & 31)] = (double)(s - 510) * 0.0067658234670659265 * env;
        }
      }
    }
  return 0;
}
