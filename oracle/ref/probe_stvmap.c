/*
 * Extracts the fixed linear maps that turn the STV building blocks
 * (Sxv[4], Syv[4], Txv[64], Tyv[64], Vv[64]; src/HEADERS/KQED.h:96-102) into
 * the 384 kernel components, by probing the reference's own hand-unrolled
 * maps with unit vectors:
 *   CONSTRUCT_FULL_KERNEL        src/LIBFILES/QED_kernel.c:16-423
 *   CONSTRUCT_KERNEL_FULL_EQZERO src/LIBFILES/QED_kernel_xy0.c:8-399
 * Both maps are linear with coefficients that are multiples of 1/4, so unit
 * probes recover them exactly.  A random-vector check confirms linearity.
 * The maps are the definition of the kernel in terms of STV; this program
 * emits them as a sparse table (C header) that the oracle and the CUDA
 * kernels share.  Test/build infrastructure only (see oracle/Makefile).
 */
#include "QED_kernel.c"
#include "QED_kernel_xy0.c"

#define NSTV 200

static void run_map(int which, const double *s, double *kp)
{
  struct STV x;
  memcpy(x.Sxv, s + 0, 4 * sizeof(double));
  memcpy(x.Syv, s + 4, 4 * sizeof(double));
  memcpy(x.Txv, s + 8, 64 * sizeof(double));
  memcpy(x.Tyv, s + 72, 64 * sizeof(double));
  memcpy(x.Vv, s + 136, 64 * sizeof(double));
  if (which == 0) CONSTRUCT_FULL_KERNEL(kp, x);
  else CONSTRUCT_KERNEL_FULL_EQZERO(kp, x);
}

static unsigned long long rng = 0x9e3779b97f4a7c15ULL;
static double urand(void)
{
  rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17;
  return (double)(rng >> 11) / 9007199254740992.0 - 0.5;
}

static int emit(int which, const char *name)
{
  static double M[384][NSTV];
  double s[NSTV], kp[384];
  int i, j, nnz = 0;
  for (j = 0; j < NSTV; j++) {
    memset(s, 0, sizeof(s));
    s[j] = 1.0;
    run_map(which, s, kp);
    for (i = 0; i < 384; i++) M[i][j] = kp[i];
  }
  /* coefficients must be multiples of 1/4 and small */
  for (i = 0; i < 384; i++)
    for (j = 0; j < NSTV; j++) {
      double q = M[i][j] * 4.0;
      if (q != (double)(long)q || fabs(q) > 127) {
        fprintf(stderr, "non-dyadic coefficient %s[%d][%d]=%g\n", name, i, j, M[i][j]);
        return 1;
      }
      if (q != 0) nnz++;
    }
  /* linearity check on random inputs */
  for (int t = 0; t < 8; t++) {
    for (j = 0; j < NSTV; j++) s[j] = urand();
    run_map(which, s, kp);
    for (i = 0; i < 384; i++) {
      double acc = 0, mag = 0;
      for (j = 0; j < NSTV; j++) { acc += M[i][j] * s[j]; mag += fabs(M[i][j] * s[j]); }
      if (fabs(acc - kp[i]) > 1e-13 * (mag + 1e-300)) {
        fprintf(stderr, "map %s not linear at row %d\n", name, i);
        return 1;
      }
    }
  }
  printf("/* %s: %d nonzeros */\n", name, nnz);
  printf("static const unsigned short %s_ROW[385] = {", name);
  int off = 0;
  for (i = 0; i <= 384; i++) {
    if (i % 16 == 0) printf("\n  ");
    printf("%d,", off);
    if (i < 384)
      for (j = 0; j < NSTV; j++) if (M[i][j] != 0) off++;
  }
  printf("\n};\n");
  printf("static const unsigned char %s_COL[%d] = {", name, nnz);
  int k = 0;
  for (i = 0; i < 384; i++)
    for (j = 0; j < NSTV; j++)
      if (M[i][j] != 0) { if (k++ % 20 == 0) printf("\n  "); printf("%d,", j); }
  printf("\n};\n");
  printf("static const signed char %s_Q4[%d] = {", name, nnz);
  k = 0;
  for (i = 0; i < 384; i++)
    for (j = 0; j < NSTV; j++)
      if (M[i][j] != 0) { if (k++ % 20 == 0) printf("\n  "); printf("%d,", (int)(M[i][j] * 4)); }
  printf("\n};\n");
  printf("#define %s_NNZ %d\n\n", name, nnz);
  return 0;
}

int main(void)
{
  printf("/* Generated by oracle/ref/probe_stvmap.c -- do not edit.\n"
         " * Sparse STV(200) -> kernel(384) maps.  STV index layout:\n"
         " *   0..3 Sx, 4..7 Sy, 8..71 Tx[a][b][d], 72..135 Ty[a][b][d], 136..199 V[a][b][d]\n"
         " * Row r lists columns COL[ROW[r]..ROW[r+1]) with coefficients Q4/4. */\n"
         "#ifndef KQED_STV_MAP_H\n#define KQED_STV_MAP_H\n\n");
  if (emit(0, "KQ_MAP_GEN")) return 1;
  if (emit(1, "KQ_MAP_ZERO")) return 1;
  printf("#endif\n");
  return 0;
}
