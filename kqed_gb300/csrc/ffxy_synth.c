/*
 * Seeded synthetic form-factor table in KQED's FFxy_single_cksum.bin format.
 *
 * The reference's real table is not distributed with its sources, so a table
 * with the same layout, checksums and loading path stands in for it.  File
 * layout (written by the reference's write_ff, src/LIBFILES/io.c:292-357, read
 * by read_ff, io.c:42-176), all little-endian:
 *   int magic=816968
 *   int nstpx, double XX[nstpx], uint32 cksum pair (rank 0)
 *   int nstpy, double YY[nstpy], uint32 cksum pair (rank 0)
 *   int Nffa
 *   Nffa x { int nstpx, nstpx x { int nstpy, nstpy x { int nf, float Fm[nf], float Fp[nf] } } }
 *   uint32 Fm_a, Fm_b, Fp_a, Fp_b   (checksum pairs, rank = running (a,ix,iy) block index)
 *
 * Grids.  XX is the reference's own x grid, recovered from its golden
 * regression files (PRECOMP/REGexample2.txt, REGexample10.txt; L0(x,0) there
 * depends only on XX and the Taylor tables): with d the TAYLORX y step,
 * XX[i] = 3(i+1) d for i <= 14 and 45 d + 9(i-14) d after, ending at 6.54 =
 * the last TAYLORX node.  The nodes are copied from the TAYLORX y grid so the
 * doubles agree exactly.  YY (uniform, the reference assumes so in its
 * second y-derivative, chnr_dV.c:460) is not recoverable; here YY[j] = 3(j+1) d
 * for j < 270, i.e. up to 6.54 with the fine x step.
 *
 * Weight functions.  For each base function b (QG0,QG1,QG2,QG3,QL4,QL2) and
 * Chebyshev index k the coefficient stored at a node is split into a y^-e_m
 * part and a y^+e_p part exactly like the reference's y-power scaling
 * (getff-new.c:110-152), so that at a node y the reconstructed value is
 *   c_k(x,y) = A_{b,k}(x) r(x,y)^k / (1+y),  r = rho * 2xy/(x^2+y^2)
 * and the reconstructed y-derivative is exactly dc_k/dy.  The x-derivative
 * tables (dxQ*, d2xQG2, d2xQG3) hold central differences of the stored
 * coefficients.  Only + - * / are used, with no contraction, so the file is
 * bit-identical on every IEEE machine.
 *
 * Usage: ffxy_synth TAYLORX_FILE OUT_FILE [seed]
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "kqed_crc32c.h"

#define NFFA 14
#define NSTPX 100
#define NSTPY 270
#define RHO 0.5

enum { QG0, QG1, QG2, QG3, QL4, QL2, dxQG0, dxQG1, dxQG2, dxQG3, dxQL4, dxQL2, d2xQG2, d2xQG3 };

static uint64_t seed_state;
static double urand_pm1(void) /* uniform in [-1,1), from a xorshift64* stream */
{
  seed_state ^= seed_state >> 12;
  seed_state ^= seed_state << 25;
  seed_state ^= seed_state >> 27;
  const uint64_t v = seed_state * 2685821657736338717ULL;
  return (double)(v >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

/* y-power exponents of the reference's scaling for base function b:
   facm_k = y^-(mshm+mm+k), facp_k = y^(mshp+mm+k)  (getff-new.c:116-146) */
static void exponents(int b, int k, int *em, int *ep)
{
  int mshm = 2;
  switch (b) {
  case QG2: mshm = 3; break;
  case QL4: mshm = 1; break;
  case QL2: mshm = 4; break;
  default: mshm = 2; break;
  }
  const int mshp = 2 - mshm;
  const int mm = mshp < 0 ? -mshp : mshp;
  *em = mshm + mm + k;
  *ep = mshp + mm + k;
}

static double ipow(double v, int e)
{
  double r = 1.0;
  int n = e < 0 ? -e : e;
  double b = v;
  while (n) {
    if (n & 1) r = r * b;
    b = b * b;
    n >>= 1;
  }
  return e < 0 ? 1.0 / r : r;
}

static double AMP[6][64];
static double SIGN[6];

/* stored Fm (which=0) or Fp (which=1) coefficient of base b at (x, y), index k */
static double coeff(int b, int k, int which, double x, double y)
{
  const double x2 = x * x, y2 = y * y;
  const double r = RHO * 2.0 * x * y / (x2 + y2);
  const double amp = SIGN[b] * AMP[b][k] * (1.0 + 0.3 * x) / (1.0 + 0.1 * x2);
  const double c = amp * ipow(r, k) / (1.0 + y);
  /* alpha = d ln c / d ln y */
  const double alpha = (double)k * (x2 - y2) / (x2 + y2) - y / (1.0 + y);
  int em, ep;
  exponents(b, k, &em, &ep);
  const double wp = (alpha + (double)em) / (double)(em + ep);
  const double wm = ((double)ep - alpha) / (double)(em + ep);
  return which == 0 ? wm * c * ipow(y, em) : wp * c * ipow(y, -ep);
}

static float to_f32(double v)
{
  if (v > 3.0e38) return 0.0f;
  if (v < -3.0e38) return 0.0f;
  return (float)v;
}

static double stored(int a, int k, int which, double x, double y)
{
  if (a < 6) return coeff(a, k, which, x, y);
  if (a < 12) {
    const double h = 1.0e-5 * x;
    const int b = a - 6;
    return (coeff(b, k, which, x + h, y) - coeff(b, k, which, x - h, y)) / (2.0 * h);
  }
  const int b = (a == d2xQG2) ? QG2 : QG3;
  const double h = 1.0e-3 * x;
  return (coeff(b, k, which, x + h, y) - 2.0 * coeff(b, k, which, x, y) +
          coeff(b, k, which, x - h, y)) / (h * h);
}

static int read_taylorx_grid(const char *path, double *g, int *n)
{
  FILE *f = fopen(path, "rb");
  if (!f) { fprintf(stderr, "ffxy_synth: cannot open %s\n", path); return 1; }
  int hdr[3];
  if (fread(hdr, sizeof(int), 3, f) != 3 || hdr[0] != 816968 || hdr[2] <= 0 || hdr[2] > 4096) {
    fprintf(stderr, "ffxy_synth: bad TAYLORX header\n");
    fclose(f);
    return 1;
  }
  *n = hdr[2];
  if (fread(g, sizeof(double), (size_t)*n, f) != (size_t)*n) { fclose(f); return 1; }
  fclose(f);
  return 0;
}

static int put(FILE *f, const void *p, size_t sz, size_t n)
{
  return fwrite(p, sz, n, f) != n;
}

int main(int argc, char **argv)
{
  if (argc < 3) {
    fprintf(stderr, "usage: %s TAYLORX_FILE OUT_FILE [seed]\n", argv[0]);
    return 2;
  }
  const uint64_t seed = argc > 3 ? strtoull(argv[3], NULL, 10) : 20240601ULL;
  seed_state = seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL;

  double tg[4096];
  int ntg = 0;
  if (read_taylorx_grid(argv[1], tg, &ntg) || ntg < 810) return 1;

  double XX[NSTPX], YY[NSTPY];
  for (int i = 0; i < NSTPX; i++) XX[i] = tg[(i <= 14 ? 3 * (i + 1) : 45 + 9 * (i - 14)) - 1];
  for (int j = 0; j < NSTPY; j++) YY[j] = tg[3 * (j + 1) - 1];
  int nfx[NSTPX];
  for (int i = 0; i < NSTPX; i++) nfx[i] = 12 + (28 * i) / (NSTPX - 1);

  for (int b = 0; b < 6; b++) {
    SIGN[b] = (b & 1) ? -1.0 : 1.0;
    for (int k = 0; k < 64; k++) AMP[b][k] = (1.0 + 0.5 * urand_pm1()) * ((k & 1) ? -0.7 : 1.0);
  }

  FILE *f = fopen(argv[2], "wb");
  if (!f) { fprintf(stderr, "ffxy_synth: cannot write %s\n", argv[2]); return 1; }
  int err = 0;
  const int magic = 816968, nx = NSTPX, ny = NSTPY, na = NFFA;
  uint32_t ck[2];
  err |= put(f, &magic, sizeof(int), 1);
  err |= put(f, &nx, sizeof(int), 1);
  err |= put(f, XX, sizeof(double), NSTPX);
  ck[0] = ck[1] = 0;
  kqed_cksum_accum(&ck[0], &ck[1], 0, XX, sizeof(XX));
  err |= put(f, ck, sizeof(uint32_t), 2);
  err |= put(f, &ny, sizeof(int), 1);
  err |= put(f, YY, sizeof(double), NSTPY);
  ck[0] = ck[1] = 0;
  kqed_cksum_accum(&ck[0], &ck[1], 0, YY, sizeof(YY));
  err |= put(f, ck, sizeof(uint32_t), 2);
  err |= put(f, &na, sizeof(int), 1);

  uint32_t ma = 0, mb = 0, pa = 0, pb = 0, rank = 0;
  float bm[64], bp[64];
  for (int a = 0; a < NFFA; a++) {
    err |= put(f, &nx, sizeof(int), 1);
    for (int i = 0; i < NSTPX; i++) {
      err |= put(f, &ny, sizeof(int), 1);
      const int nf = nfx[i];
      for (int j = 0; j < NSTPY; j++) {
        for (int k = 0; k < nf; k++) {
          bm[k] = to_f32(stored(a, k, 0, XX[i], YY[j]));
          bp[k] = to_f32(stored(a, k, 1, XX[i], YY[j]));
        }
        err |= put(f, &nf, sizeof(int), 1);
        err |= put(f, bm, sizeof(float), (size_t)nf);
        kqed_cksum_accum(&ma, &mb, rank, bm, (size_t)nf * sizeof(float));
        err |= put(f, bp, sizeof(float), (size_t)nf);
        kqed_cksum_accum(&pa, &pb, rank, bp, (size_t)nf * sizeof(float));
        rank++;
      }
    }
  }
  const uint32_t tail[4] = {ma, mb, pa, pb};
  err |= put(f, tail, sizeof(uint32_t), 4);
  err |= fclose(f) != 0;
  if (err) { fprintf(stderr, "ffxy_synth: write error\n"); return 1; }
  printf("%08x %08x %08x %08x\n", ma, mb, pa, pb);
  return 0;
}
