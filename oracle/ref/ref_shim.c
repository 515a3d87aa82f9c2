/*
 * Thin wrapper compiled together with the reference KQED library sources
 * (test infrastructure only; see oracle/Makefile).  It gives ctypes a flat
 * interface to the reference's own QED_kernel_L0..L3
 * (src/LIBFILES/kernels.c:82-177) and initialise/free_QED_temps
 * (src/LIBFILES/init.c:38,142), without re-declaring struct QED_kernel_temps
 * on the Python side.
 */
#include "KQED.h"

#include <omp.h>

const char *kqedref_lib_path(void)
{
  const char *p = getenv("KQEDREF_PATH");
  return p ? p : ".";
}

static struct QED_kernel_temps T;
static int T_ready = 0;
/* the reference sizes its per-thread scratch by omp_get_max_threads() at
   initialise (src/LIBFILES/init.c:119,178) and indexes it by thread number
   in the kernels (src/LIBFILES/QED_kernel.c:449): no call may run more
   threads than this */
static int T_threads = 0;

int ref_init(void)
{
  if (T_ready) return 0;
  memset(&T, 0, sizeof(T));
  T_threads = omp_get_max_threads();
  if (initialise(&T)) return 1;
  T_ready = 1;
  return 0;
}

/* ref_init with the reference's scratch sized for nthreads threads
   (whatever OMP_NUM_THREADS says); no effect once initialised */
int ref_init_threads(int nthreads)
{
  if (!T_ready && nthreads > 0) omp_set_num_threads(nthreads);
  return ref_init();
}

void ref_free(void)
{
  if (!T_ready) return;
  free_QED_temps(&T);
  memset(&T, 0, sizeof(T));
  T_ready = 0;
}

int ref_grid_info(int *nstpx, int *nstpy, int *nffa, double *xlo, double *xhi,
                  double *ylo, double *yhi)
{
  if (!T_ready) return 1;
  *nstpx = T.Grid.nstpx; *nstpy = T.Grid.nstpy; *nffa = T.Grid.Nffa;
  *xlo = T.Grid.XX[0]; *xhi = T.Grid.XX[T.Grid.nstpx - 1];
  *ylo = T.Grid.YY[0]; *yhi = T.Grid.YY[T.Grid.nstpy - 1];
  return 0;
}

typedef void (*kfun)(const double *, const double *, const struct QED_kernel_temps,
                     double[6][4][4][4]);

static kfun pick(int variant)
{
  switch (variant) {
  case 0: return (kfun)QED_kernel_L0;
  case 1: return (kfun)QED_kernel_L1;
  case 2: return (kfun)QED_kernel_L2;
  case 3: return (kfun)QED_kernel_L3;
  default: return NULL;
  }
}

/* out[n][384]; pairs spread over OpenMP threads like the reference's own
   stress test (src/amu_forlattice.c:1419-1429). */
int ref_kernel(int variant, long n, const double *x, const double *y, double *out,
               int nthreads)
{
  kfun f = pick(variant);
  if (!T_ready || !f) return 1;
  if (nthreads <= 0 || nthreads > T_threads) nthreads = T_threads;
  long i;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (i = 0; i < n; i++) {
    double kerv[6][4][4][4] KQED_ALIGN;
    f(x + 4 * i, y + 4 * i, T, kerv);
    memcpy(out + 384 * i, kerv, 384 * sizeof(double));
  }
  return 0;
}

/* Fused lattice contraction sum_i L_i(x,y) Pi_i(x,y) over n pairs, the way
   the reference's example driver contracts a kernel with pihat
   (src/amu_forlattice.c:100-108).  Returns the per-pair dot products. */
int ref_contract(int variant, long n, const double *x, const double *y,
                 const double *pi, double *dots, int nthreads)
{
  kfun f = pick(variant);
  if (!T_ready || !f) return 1;
  if (nthreads <= 0 || nthreads > T_threads) nthreads = T_threads;
  long i;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (i = 0; i < n; i++) {
    double kerv[6][4][4][4] KQED_ALIGN;
    f(x + 4 * i, y + 4 * i, T, kerv);
    const double *k = (const double *)kerv;
    const double *p = pi + 384 * i;
    double s = 0.0;
    int c;
    for (c = 0; c < 384; c++) s += k[c] * p[c];
    dots[i] = s;
  }
  return 0;
}

/* The reference's composite kernels (src/LIBFILES/all_kernels.c,
   con_kernel.c, sub_kernel.c, SYMXY.c, SYMXY0.c, kernels.c:181-231) over n
   pairs, each pair's output struct copied to out[i][size]; `which` numbers
   them as the oracle does (oracle_composite). */
long ref_composite_size(int which)
{
  switch (which) {
  case 0: case 1: case 2: case 3: case 7: case 9: return 3072;
  case 4: case 5: case 6: return 4608;
  case 8: case 10: return 1536;
  case 11: return 384;
  default: return 0;
  }
}

int ref_composite(int which, const double *M, long n, const double *x, const double *y,
                  double *out, int nthreads)
{
  const long sz = ref_composite_size(which);
  if (!T_ready || sz == 0) return 1;
  if (nthreads <= 0 || nthreads > T_threads) nthreads = T_threads;
  long i;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
  for (i = 0; i < n; i++) {
    const double *xv = x + 4 * i, *yv = y + 4 * i;
    double *o = out + sz * i;
    struct QED_Kernels Q;
    struct Kernels K[3];
    double kerv[6][4][4][4] KQED_ALIGN;
    switch (which) {
    case 0: compute_all_kernels(xv, yv, T, &Q); memcpy(o, &Q, sizeof(Q)); break;
    case 1: compute_all_Mkernels(M, xv, yv, T, &Q); memcpy(o, &Q, sizeof(Q)); break;
    case 2: compute_all_Mkernels_v2(M, xv, yv, T, &Q); memcpy(o, &Q, sizeof(Q)); break;
    case 3: compute_con_kernels(xv, yv, T, &Q); memcpy(o, &Q, sizeof(Q)); break;
    case 4: compute_con_kernels_v2(xv, yv, T, K); memcpy(o, K, sizeof(K)); break;
    case 5: compute_con_kernelsM_L2(M, xv, yv, T, K); memcpy(o, K, sizeof(K)); break;
    case 6: compute_sub_kernelsM_L2(M, xv, yv, T, K); memcpy(o, K, sizeof(K)); break;
    case 7: compute_all_kernels_SYMXY(xv, yv, T, &Q); memcpy(o, &Q, sizeof(Q)); break;
    case 8: compute_all_kernels_SYMXY_v2(xv, yv, T, K); memcpy(o, K, sizeof(K[0])); break;
    case 9: compute_all_kernels_SYMXY0(xv, yv, T, &Q); memcpy(o, &Q, sizeof(Q)); break;
    case 10: compute_all_kernels_SYMXY0_v2(xv, yv, T, K); memcpy(o, K, sizeof(K[0])); break;
    case 11: QED_Mkernel_L2(M[0], xv, yv, T, kerv); memcpy(o, kerv, sizeof(kerv)); break;
    }
  }
  return 0;
}

/* the reference's perturbative Pi-hat, ipihatFermLoop_antisym
   (src/LIBFILES/pi_pert.c:162-198), over n pairs: out[n][384] */
int ref_pihat(long n, const double *x, const double *y, double *out, int nthreads)
{
  if (!T_ready) return 1;
  if (nthreads <= 0 || nthreads > T_threads) nthreads = T_threads;
  long i;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
  for (i = 0; i < n; i++) {
    double v[6][4][4][4];
    ipihatFermLoop_antisym(x + 4 * i, y + 4 * i, T, v);
    memcpy(out + 384 * i, v, sizeof(v));
  }
  return 0;
}

/* the reference's G8 table as initialise() filled it */
int ref_g8(int *out)
{
  if (!T_ready || !T.G8) return 1;
  memcpy(out, T.G8, 65536 * sizeof(int));
  return 0;
}

/* the reference's one-loop tensor pihat1 (pi_pert.c:236-389) of one pair:
   out[1024 + 256] = vpihat1 then vpihatr1 */
int ref_pihat1(const double *x, const double *y, double *out)
{
  if (!T_ready) return 1;
  double p[4][4][4][4][4], r[4][4][4][4];
  pihat1(x, y, T, p, r);
  memcpy(out, p, sizeof(p));
  memcpy(out + 1024, r, sizeof(r));
  return 0;
}
