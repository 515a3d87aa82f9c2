/*
 * ORACLE -- test infrastructure only.
 *
 * A CPU restatement, in plain C, of the reference KQED library's kernel path
 * (QED_kernel_L0..L3 and everything beneath them), following the reference's
 * portable (non-AVX) code path step for step.  It is the checker for the CUDA
 * implementation: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The product never calls it.
 *
 * Parity is pinned three ways: against the reference library compiled from its
 * own sources (oracle/Makefile), against the reference's golden regression
 * files for the table-independent branches (PRECOMP/REGexample2.txt,
 * REGexample10.txt), and through the reference's identity tests.
 */
#ifndef KQED_ORACLE_H
#define KQED_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Loads LIB_PATH/PRECOMP/{FFxy_single_cksum,taylorx_cksum,taylory_cksum}.bin
   with checksum validation.  Returns 0 on success. */
int oracle_load(const char *lib_path);
void oracle_free(void);
int oracle_grid(int *nstpx, int *nstpy, double *xlo, double *xhi, double *ylo, double *yhi);

/* out[n][384] = QED_kernel_L<variant>(x[i], y[i]); variant 0..3. */
int oracle_kernel(int variant, long n, const double *x, const double *y, double *out,
                  int nthreads);

/* out[384] = QED_kernel_L0(xv, yv); 0 on success */
int oracle_L0_one(const double xv[4], const double yv[4], double *out);

/* The reference's composite kernels (src/LIBFILES/all_kernels.c,
   con_kernel.c, sub_kernel.c, SYMXY.c, SYMXY0.c, kernels.c:181-231),
   restated in kqed_composite_oracle.c.  `which` numbers them as enum
   kqed_composite of the library's C ABI; out[n][oracle_composite_size(which)]
   holds each pair's output struct (struct Kernels, struct QED_Kernels,
   struct Kernels[3] or one kernel) in the reference's memory layout.  M:
   the four masses of the M-subtracted forms, M[0] alone for QED_Mkernel_L2,
   ignored otherwise. */
long oracle_composite_size(int which);
int oracle_composite(int which, const double *M, long n, const double *x, const double *y,
                     double *out, int nthreads);

/* The perturbative lepton-loop Pi-hat of the reference
   (ipihatFermLoop_antisym, src/LIBFILES/pi_pert.c:162-198), restated in
   kqed_pihat_oracle.c: out[n][6][4][4][4]; and the Dirac-trace table G8
   (init_g8, pi_pert.c:140-160) into out[65536]. */
int oracle_pihat(long n, const double *x, const double *y, double *out, int nthreads);
int oracle_g8(int *out);

/* dots[i] = sum_c L<variant>_c(x[i],y[i]) * pi[i][c] */
int oracle_contract(int variant, long n, const double *x, const double *y, const double *pi,
                    double *dots, int nthreads);

/* out[n][200]: the STV building blocks (Sx, Sy, Tx, Ty, V) of generic pairs */
int oracle_stv(long n, const double *x, const double *y, double *out);

/* Branch taken by L0(x,y): 0 zero (x=y=0), 1 x=0, 2 y=0, 3 x=y, 4 generic,
   5 generic with |x| below the grid (Taylor in x); +8 if the x<->(x-y) swap is
   active; 16 if the kernel is zero because an argument is outside the grid. */
int oracle_branch(long n, const double *x, const double *y, int *code);

/* The 37 interpolated weight-function values of a generic pair, evaluated at
   the post-swap invariants (|x|, |y|, cb) inside the grid: the inputs of the
   learned surrogate.  out[n][37]; returns 0. */
int oracle_weights(long n, const double *X, const double *Y, const double *CB, double *out,
                   int nthreads);

/* The synthetic Pi of kqed_lattice_sum_synth / kqed_pi_synth_dev (a
   benchmark input): pi[nx][ny][384] for x indices k0 .. k0 + nx - 1 and
   site indices n0 .. n0 + ny - 1. */
int oracle_pi_synth(long nx, const double *x, long ny, const double *y, uint64_t seed,
                    uint32_t stream, long k0, long n0, double *pi);

#ifdef __cplusplus
}
#endif

#endif
