/*
 * kqed.h -- C ABI of libkqed_gb300.so, a GB300 (sm_103a) evaluator of KQED's
 * position-space QED kernel L^{(0..3)}_{[rho sigma]; mu nu lambda}(x, y).
 *
 * Part 1 is a drop-in for the reference library's kernel API: the same
 * structs (field order and sizes unchanged), the same function names,
 * argument meaning, table files and error behaviour.  A lattice code that
 * includes the reference's KQED.h and links this library instead gets the
 * kernel evaluated on the GPU.
 *
 * Part 2 adds batched and fused entry points that carry the throughput.
 * All pointers are plain host or device pointers; no library types appear in
 * the signatures.  Return value 0 means success; a positive value is an error
 * code and kqed_last_error() gives the message for the calling thread.
 */
#ifndef KQED_GB300_H
#define KQED_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------
 * Part 1: reference-compatible API
 * ---------------------------------------------------------------------- */

/* src/HEADERS/KQED.h:63-67 of the reference.  In this library `Fm` holds the
   opaque device context and `Fp`, `nmax` are unused. */
struct AVX_precomps {
  void *Fm, *Fp;
  int nmax;
};

/* src/HEADERS/KQED.h:69-87.  initialise() fills every field exactly as the
   reference does (grids, ragged Ffm/Ffp coefficient arrays, Taylor tables);
   PC points at the library's device context. */
struct Grid_coeffs {
  int Nffa;
  float ****Ffp;
  float ****Ffm;
  double *XX;
  double *YY;
  double xstp;
  double ystp;
  int nstpx;
  int nstpy;
  double **TX; /* [23][NY_tay] */
  int NtayX;
  int NY_tay;
  double **TY; /* [14][NX_tay] */
  int NtayY;
  int NX_tay;
  struct AVX_precomps *PC;
  int *nfx;
};

/* src/HEADERS/KQED.h:90-93.  G8: the 65,536-entry Dirac-trace table of the
   perturbative lepton-loop Pi-hat, filled by initialise() as the
   reference's (init_g8) and freed by free_QED_temps(). */
struct QED_kernel_temps {
  struct Grid_coeffs Grid;
  int *G8;
};

/* Replaces initialise(), src/LIBFILES/init.c:142 (declared src/HEADERS/init.h:7).
   Reads LIB_PATH/PRECOMP/{FFxy_single_cksum,taylorx_cksum,taylory_cksum}.bin,
   validates their CRC32C checksums, and uploads the tables to the GPU.
   LIB_PATH is the environment variable KQED_LIB_PATH if set, else the
   directory the library was built in.  Returns 1 on failure with a message
   on stderr, 0 on success. */
int initialise(struct QED_kernel_temps *t);

/* Alias with the name used in the project description. */
int initialize_QED_kernel_temps(struct QED_kernel_temps *t);

/* Replaces free_QED_temps(), src/LIBFILES/init.c:38 (src/HEADERS/init.h:4). */
void free_QED_temps(struct QED_kernel_temps *t);

/* Replace the table readers and writers of src/LIBFILES/io.c:42-412
   (src/HEADERS/io.h:4-20).  The readers fill the Grid fields from
   LIB_PATH/PRECOMP with checksum validation (0 on success, 1 with a message
   on stderr); initialise() calls the same code.  The writers produce the
   same checksummed files under ./PRECOMP of the working directory:
   FFxy_single_cksum2.bin, taylorx_cksum.bin, taylory_cksum.bin. */
int read_ff(struct Grid_coeffs *Grid);
int read_TAYLORX(struct Grid_coeffs *Grid);
int read_TAYLORY(struct Grid_coeffs *Grid);
void write_ff(const struct Grid_coeffs *Grid);
void write_TAYLORX(const struct Grid_coeffs *Grid);
void write_TAYLORY(const struct Grid_coeffs *Grid);

/* Replace QED_kernel_L0..L3, src/LIBFILES/kernels.c:81-177
   (src/HEADERS/kernels.h:4-33).  kerv is fully overwritten; a pair outside
   the tabulated grid gives an all-zero kernel, as in the reference.
   Thread-safe: concurrent callers each get their own stream and staging. */
void QED_kernel_L0(const double xv[4], const double yv[4], const struct QED_kernel_temps t,
                   double kerv[6][4][4][4]);
void QED_kernel_L1(const double xv[4], const double yv[4], const struct QED_kernel_temps t,
                   double kerv[6][4][4][4]);
void QED_kernel_L2(const double xv[4], const double yv[4], const struct QED_kernel_temps t,
                   double kerv[6][4][4][4]);
void QED_kernel_L3(const double xv[4], const double yv[4], const struct QED_kernel_temps t,
                   double kerv[6][4][4][4]);

/* src/HEADERS/KQED.h:101-125: the composite kernels' output structs (the
   reference aligns their arrays to 32 bytes in AVX builds; the layout --
   sizes and offsets -- is the same either way). */
struct Kernel {
  double xy[6][4][4][4];
  double yx[6][4][4][4];
};
struct Kernels {
  double L0[6][4][4][4];
  double L1[6][4][4][4];
  double L2[6][4][4][4];
  double L3[6][4][4][4];
};
struct QED_Kernels {
  struct Kernel L0;
  struct Kernel L1;
  struct Kernel L2;
  struct Kernel L3;
};
struct QED_Con_Kernels {
  struct Kernels A;
  struct Kernels B;
  struct Kernels C;
};

/* Replace QED_Mkernel_L2, src/LIBFILES/kernels.c:181-231 (kernels.h:23-28):
   L0(x,y) - exp(-M x^2/2)[L0(0,y) - M x_mu x.L0(0,y)]
           - exp(-M y^2/2)[L0(x,0) - M y_nu y.L0(x,0)]. */
void QED_Mkernel_L2(const double M, const double xv[4], const double yv[4],
                    const struct QED_kernel_temps t, double kerv[6][4][4][4]);

/* Replace the composite kernels of src/LIBFILES/all_kernels.c, con_kernel.c,
   sub_kernel.c, SYMXY.c and SYMXY0.c (declared in src/HEADERS/all_kernels.h,
   con_kernel.h, sub_kernel.h, SYMXY.h, SYMXY0.h): the same combinations of
   L0 at derived arguments, evaluated on the GPU (kqed_composite_batch below
   is the batched form).  Outputs fully overwritten; on an error a message
   goes to stderr and the output is zero. */
void compute_all_kernels(const double xv[4], const double yv[4], const struct QED_kernel_temps t,
                         struct QED_Kernels *K);
void compute_all_Mkernels(const double M[4], const double xv[4], const double yv[4],
                          const struct QED_kernel_temps t, struct QED_Kernels *K);
void compute_all_Mkernels_v2(const double M[4], const double xv[4], const double yv[4],
                             const struct QED_kernel_temps t, struct QED_Kernels *K);
void compute_con_kernels(const double xv[4], const double yv[4], const struct QED_kernel_temps t,
                         struct QED_Kernels *K);
void compute_con_kernels_v2(const double xv[4], const double yv[4],
                            const struct QED_kernel_temps t, struct Kernels *K);
void compute_con_kernelsM_L2(const double M[4], const double xv[4], const double yv[4],
                             const struct QED_kernel_temps t, struct Kernels *K);
void compute_sub_kernelsM_L2(const double M[4], const double xv[4], const double yv[4],
                             const struct QED_kernel_temps t, struct Kernels *K);
void compute_all_kernels_SYMXY(const double xv[4], const double yv[4],
                               const struct QED_kernel_temps t, struct QED_Kernels *K);
void compute_all_kernels_SYMXY_v2(const double xv[4], const double yv[4],
                                  const struct QED_kernel_temps t, struct Kernels *K);
void compute_all_kernels_SYMXY0(const double xv[4], const double yv[4],
                                const struct QED_kernel_temps t, struct QED_Kernels *K);
void compute_all_kernels_SYMXY0_v2(const double xv[4], const double yv[4],
                                   const struct QED_kernel_temps t, struct Kernels *K);
/* host helpers of the same files: K = (K + W)/2 (all_kernels.c:19-82,
   con_kernel.c:14-59, over K[0..2]) and mu <-> nu on every L<i>.yx
   (all_kernels.c:373-406) */
void average_all_kernels(struct Kernels *K, const struct Kernels W);
void average_all_QED_kernels(struct QED_Kernels *K, const struct QED_Kernels W);
void average_con_kernels(struct Kernels *K, const struct Kernels *W);
void swap_munu_Lyx(struct QED_Kernels *K);

/* Replace the perturbative lepton-loop functions of src/LIBFILES/pi_pert.c
   (src/HEADERS/pi_pert.h): the (rho, sigma)-antisymmetrised Pi-hat of a
   free lepton loop, and the one-loop tensor it is built from, evaluated on
   the GPU (kqed_pihat_batch below is the batched form); the Dirac traces,
   the Bessel functions K_0..K_n and the analytic a_mu and vacuum-
   polarisation results, on the host.  The analytic functions print nothing
   (the reference prints its partial sums). */
void ipihatFermLoop_antisym(const double x[4], const double y[4], const struct QED_kernel_temps t,
                            double vpihat[6][4][4][4]);
void pihat1(const double x[4], const double y[4], const struct QED_kernel_temps t,
            double vpihat1[4][4][4][4][4], double vpihatr1[4][4][4][4]);
void init_g8(struct QED_kernel_temps *t);
int diractrace(const int n, const int *idx);
void bessk(const int n, const double x, double *bv);
double amu_heavlept(const double mh);
double amu_lightlept(const double ml);
double vac_pol(const double ml);

/* ------------------------------------------------------------------------
 * Part 2: batched and fused entry points (no counterpart in the reference's
 * library; they replace the caller-side loop of src/amu_forlattice.c:1419-1429
 * and the contraction of src/amu_forlattice.c:100-108)
 * ---------------------------------------------------------------------- */

enum kqed_precision {
  KQED_FP64 = 0,        /* plain FP64 throughout */
  KQED_FP32_MIXED = 1,  /* FP32 interpolation/assembly, FP64 where stability needs it */
  KQED_SURROGATE = 2    /* learned weight functions with interpolation fallback */
};

/* Per-pair status bits written by the batched calls when status != NULL. */
enum kqed_status_bits {
  KQED_ST_OK = 0,
  KQED_ST_OUT_OF_GRID = 1, /* kernel set to zero, as the reference does */
  KQED_ST_TAYLOR_X = 2,    /* |x| below the first grid node: Taylor branch */
  KQED_ST_SWAP = 4,        /* x <-> (x - y) swap branch */
  KQED_ST_AXIS = 8         /* x = 0, y = 0 or x = y special form */
};

/* kerv[i][384] = QED_kernel_L<variant>(x[i], y[i]) for i < n, host buffers
   (x, y: n*4 doubles; kerv: n*384 doubles; status: n bytes or NULL).  A
   kerv lying wholly inside one allocation of kqed_pinned_alloc is written
   in place by the kernels (no device copy); the values are the same. */
int kqed_kernel_batch(const struct QED_kernel_temps *t, int variant, size_t n, const double *x,
                      const double *y, double *kerv, uint8_t *status, int precision);

/* Same with device pointers, enqueued on `stream` (a cudaStream_t, NULL for
   the legacy default stream); returns after enqueueing. */
int kqed_kernel_batch_dev(const struct QED_kernel_temps *t, int variant, size_t n,
                          const double *d_x, const double *d_y, double *d_kerv,
                          uint8_t *d_status, int precision, void *stream);

/* The composite kernels, batched.  Numbering and per-pair output (the
   reference's struct, in its memory layout):
     KQED_ALL_KERNELS      compute_all_kernels            struct QED_Kernels
     KQED_ALL_MKERNELS     compute_all_Mkernels (M[4])    struct QED_Kernels
     KQED_ALL_MKERNELS_V2  compute_all_Mkernels_v2 (M[4]) struct QED_Kernels
     KQED_CON_KERNELS      compute_con_kernels            struct QED_Kernels
     KQED_CON_KERNELS_V2   compute_con_kernels_v2         struct Kernels[3]
     KQED_CON_KERNELSM_L2  compute_con_kernelsM_L2 (M[4]) struct Kernels[3]
     KQED_SUB_KERNELSM_L2  compute_sub_kernelsM_L2 (M[4]) struct Kernels[3]
     KQED_SYMXY            compute_all_kernels_SYMXY      struct QED_Kernels
     KQED_SYMXY_V2         compute_all_kernels_SYMXY_v2   struct Kernels
     KQED_SYMXY0           compute_all_kernels_SYMXY0     struct QED_Kernels
     KQED_SYMXY0_V2        compute_all_kernels_SYMXY0_v2  struct Kernels
     KQED_MKERNEL_L2       QED_Mkernel_L2 (M[0])          double[6][4][4][4] */
enum kqed_composite {
  KQED_ALL_KERNELS = 0,
  KQED_ALL_MKERNELS = 1,
  KQED_ALL_MKERNELS_V2 = 2,
  KQED_CON_KERNELS = 3,
  KQED_CON_KERNELS_V2 = 4,
  KQED_CON_KERNELSM_L2 = 5,
  KQED_SUB_KERNELSM_L2 = 6,
  KQED_SYMXY = 7,
  KQED_SYMXY_V2 = 8,
  KQED_SYMXY0 = 9,
  KQED_SYMXY0_V2 = 10,
  KQED_MKERNEL_L2 = 11,
  KQED_COMPOSITE_COUNT = 12
};

/* doubles per pair of a composite's output (0 for an unknown one) */
size_t kqed_composite_size(int which);

/* out[i][kqed_composite_size(which)] = composite `which` at (x[i], y[i]) for
   i < n.  M: host pointer to the masses (4 doubles; 1 for
   KQED_MKERNEL_L2), NULL for the forms without masses.  precision:
   KQED_FP64 or KQED_FP32_MIXED (the form of the L0 evaluations; the
   combinations are FP64).  Host buffers; an out lying wholly inside one
   allocation of kqed_pinned_alloc is written in place by the kernels. */
int kqed_composite_batch(const struct QED_kernel_temps *t, int which, const double *M, size_t n,
                         const double *x, const double *y, double *out, int precision);

/* Same with device pointers (M stays a host pointer), enqueued on `stream`. */
int kqed_composite_batch_dev(const struct QED_kernel_temps *t, int which, const double *M,
                             size_t n, const double *d_x, const double *d_y, double *d_out,
                             int precision, void *stream);

/* out[i][384] = ipihatFermLoop_antisym(x[i], y[i]) for i < n: host buffers,
   or device buffers enqueued on `stream`. */
int kqed_pihat_batch(size_t n, const double *x, const double *y, double *out);
int kqed_pihat_batch_dev(size_t n, const double *d_x, const double *d_y, double *d_out,
                         void *stream);
/* d_pi[k][n][384] = ipihatFermLoop_antisym(scale x_k, scale y_n): the
   perturbative Pi-hat of a lepton of mass `scale` (in units of the kernel's
   mass) laid out as the fused lattice sums take it (the reference's
   lepton-loop check, src/amu_forlattice.c:65-116, uses scale = 2). */
int kqed_pihat_lattice_dev(size_t nx, const double *d_x, size_t ny, const double *d_y,
                           double scale, double *d_pi, void *stream);

/* Fused lattice integrand.  For each of nx points x_k and all ny sites y_n:
     sums[k] = sum_n sum_c L<variant>_c(x_k, y_n) * pi[k][n][c]
   with pi laid out [nx][ny][384].  Accumulation is FP64 with compensated
   (Neumaier) summation and a fixed reduction order, so results are
   reproducible.  An empty lattice (ny = 0) gives zero sums; its site and pi
   pointers may then be NULL.  Host buffers.  A pi lying wholly inside one
   allocation of kqed_pinned_alloc is read in place by the kernels over the
   host link (no staging copies); any other pi is copied to the device in
   chunks overlapped with the kernels.  The sums are the same either way;
   the environment variable KQED_HOST_PI=copy forces the copies. */
int kqed_lattice_sum(const struct QED_kernel_temps *t, int variant, size_t nx, const double *x,
                     size_t ny, const double *y, const double *pi, double *sums, int precision);

/* Same with device pointers on `stream`; d_sums must hold nx doubles.  The
   library's device scratch for these calls is per host thread (the mixed
   form also runs part of the work on a stream of that thread, joined back
   to `stream` by events): calls from one thread on different streams must
   not overlap on the device (order the streams, e.g. with an event); calls
   from different threads are independent. */
int kqed_lattice_sum_dev(const struct QED_kernel_temps *t, int variant, size_t nx,
                         const double *d_x, size_t ny, const double *d_y, const double *d_pi,
                         double *d_sums, int precision, void *stream);

/* The fused lattice sum for callers that cannot allocate GPU memory (codes
   whose own pool owns the device; loops where cudaMalloc's implicit device
   synchronisation would stall other streams).  It has no counterpart in the
   reference.  Same arguments as kqed_lattice_sum_dev (FP64 form only), and
   the same reduction order; results agree with it to about 1e-12 relative,
   not bit for bit, because without room for per-x column tables the record
   kernel interpolates from the node table, as the pair batches do.  Its
   scratch comes from a static 16 MiB device array compiled into the library
   (held by every GPU that loads it), so problems needing more scratch are
   rejected with an error: nx * ceil(ny / 64) * 2 doubles, plus, for L1..L3,
   388 * ny + 772 * nx doubles, plus one tile of pair records (64 * 88 + 8
   doubles), must not exceed 2,097,152.  The first call in a CUDA context
   (once per device, and again after cudaDeviceReset) looks up the array's
   device address; make it before any stream capture.  Calls share the
   array: calls that overlap on the GPU race and must be serialised by the
   caller.  Allocates nothing. */
int kqed_lattice_sum_noalloc(const struct QED_kernel_temps *t, int variant, size_t nx,
                             const double *d_x, size_t ny, const double *d_y, const double *d_pi,
                             double *d_sums, void *stream);

/* Synthetic Pi for benchmark lattices too large to hold Pi in memory (no
   reference counterpart; the reference's callers supply Pi).  Component c
   of Pi(x_k, y_n), k the index of x in d_x, is
     g * exp(-(|y_n| + |x_k - y_n|) / 2),
     g = (b0 + b1 + b2 + b3 - 510) * sqrt(3) / 256,
   b0..b3 the bytes of word (c >> 5) & 3 of Philox-4x32-10 with key seed
   (low word first) and counter (y_offset + n, x_offset + k,
   (c & 31) + 32 * (c >> 7), stream_id): mean 0, variance 1 - 2^-16.  The
   offsets are the global indices of d_x[0] and d_y[0], so a lattice split
   into slabs of sites (or of x points) sees the same Pi in every piece.
   kqed_lattice_sum_synth: the fused lattice sum with this Pi generated inside
   the kernel (nothing of Pi is stored); otherwise as kqed_lattice_sum_dev.
   kqed_pi_synth_dev: the same Pi written to d_pi [nx][ny][384]. */
int kqed_lattice_sum_synth(const struct QED_kernel_temps *t, int variant, size_t nx,
                           const double *d_x, size_t ny, const double *d_y, uint64_t seed,
                           uint32_t stream_id, size_t x_offset, size_t y_offset, double *d_sums,
                           int precision, void *stream);
int kqed_pi_synth_dev(size_t nx, const double *d_x, size_t ny, const double *d_y, uint64_t seed,
                      uint32_t stream_id, size_t x_offset, size_t y_offset, double *d_pi,
                      void *stream);

/* Page-locked, device-mapped host memory (cudaHostAlloc) for the inputs of
   the host entry points, e.g. the caller's Pi of kqed_lattice_sum, which the
   kernels then read in place.  Free with kqed_pinned_free.
   kqed_pinned_contains: 1 if [ptr, ptr + bytes) lies wholly inside one live
   allocation of kqed_pinned_alloc, else 0. */
int kqed_pinned_alloc(size_t bytes, void **ptr);
int kqed_pinned_free(void *ptr);
int kqed_pinned_contains(const void *ptr, size_t bytes);

/* Multi-GPU sharding of a lattice sum, one process per GPU: rank `rank` of
   `world` takes sites [*begin, *end) (contiguous slabs of whole 64-site
   tiles) and evaluates them against all x -- kqed_lattice_sum_dev on its
   slab of sites and Pi, or kqed_lattice_sum_synth with y_offset = *begin;
   the caller gathers the nx partial sums of every rank (one MPI_Allgather /
   ncclAllGather of nx doubles) into parts[world][nx], and
   kqed_shard_combine adds them in rank order with compensated summation. */
int kqed_shard_slab(size_t ny, int rank, int world, size_t *begin, size_t *end);
int kqed_shard_combine(size_t nx, int world, const double *parts, double *sums);

/* Message of the last error on the calling thread ("" if none). */
const char *kqed_last_error(void);

/* Number of this library's GPU kernels launched so far by this process. */
uint64_t kqed_launch_count(void);

/* Batched lattices (no reference counterpart): many fused lattice sums as
   one work list, captured once in a CUDA graph and replayed.
   kqed_batch_plan_create allocates everything the batch needs, runs it once
   (with tune != 0 it first times candidate launch parameters -- assembly
   warps per block, assembly grid, record chunk -- on this batch's first
   131,072 units (8.4 M pairs) and keeps
   the fastest, remembered per device, precision and batch size), then
   captures the batch -- column tables, kernel terms, the record and
   assembly kernels over all jobs' units, the per-job reductions -- in a CUDA
   graph.  kqed_batch_plan_launch replays the graph on `stream`: each job's
   d_sums[k] = sum_y L<variant>(x_k, y).Pi(x_k, y) for the current contents
   of its buffers (the pointers are fixed at creation).  A job's d_pi NULL
   selects the generated Pi of kqed_lattice_sum_synth with its
   (pi_seed, pi_stream). */
struct kqed_lattice_job {
  int variant;            /* 0..3 */
  size_t nx, ny;
  const double *d_x;      /* [nx][4] device */
  const double *d_y;      /* [ny][4] device */
  const double *d_pi;     /* [nx][ny][384] device, or NULL (generated) */
  uint64_t pi_seed;
  uint32_t pi_stream;
  double *d_sums;         /* [nx] device */
};
struct kqed_batch_info {
  int jobs;
  size_t units;           /* (x, 64-site tile) work units of the batch */
  size_t pairs;           /* (x, y) evaluations per launch */
  int warps_per_block;    /* launch parameters in the graph */
  int blocks;             /* 0: one persistent grid at full occupancy */
  size_t record_chunk_pairs;
  size_t graph_kernels;   /* kernel nodes in the graph */
  double tuned_ms;        /* best time of the main kernels while tuning, or 0 */
};
typedef struct kqed_batch_plan kqed_batch_plan;
int kqed_batch_plan_create(const struct QED_kernel_temps *t, int njobs,
                           const struct kqed_lattice_job *jobs, int precision, int tune,
                           kqed_batch_plan **plan);
int kqed_batch_plan_launch(kqed_batch_plan *plan, void *stream);
int kqed_batch_plan_info(const kqed_batch_plan *plan, struct kqed_batch_info *info);
void kqed_batch_plan_destroy(kqed_batch_plan *plan);

/* Error of the mixed-precision form against the plain FP64 form on n pairs
   (device buffers d_x, d_y [n][4]), accumulated on the device; no reference
   counterpart.  For every pair with a nonzero kernel, norm = max_c |L_c|
   (FP64 form) and r_c = |L_c(mixed) - L_c(FP64)| / max(norm, floor_abs).
   On return (host buffer of KQED_STATS_LEN doubles):
     stats[c]        max over pairs of r_c,          c = 0..383
     stats[384 + c]  root mean square over pairs of r_c
     stats[768]      max over pairs of max_c r_c
     stats[769]      mean over pairs of max_c r_c
     stats[770]      number of pairs counted
   Runs on `stream` and synchronises it before returning. */
#define KQED_STATS_LEN 771
int kqed_precision_stats(const struct QED_kernel_temps *t, int variant, size_t n,
                         const double *d_x, const double *d_y, double floor_abs, double *stats,
                         void *stream);

/* The learned surrogate (precision KQED_SURROGATE; no reference
   counterpart).  A 3 -> 256 -> 256 -> 256 -> 39 MLP (SiLU) maps a generic
   pair's post-swap invariants (|x|, |y|, cb) to the 39 weight functions that
   the reference interpolates from its form-factor grid (extractff2 / getff7,
   src/LIBFILES/getff-new.c:262-312, src/LIBFILES/simd.c:488-612).  It is
   trained on the GPU by this library's own BF16 tensor-core kernels (FP32
   accumulation) on samples labelled by the FP64 interpolation, and attached
   to the tables `t`; the lattice entry points with precision KQED_SURROGATE
   then evaluate it wherever the held-out error bound of a pair's cell of
   (ln|x|, ln|y|, cb) is <= tau, and fall back to the interpolation (the
   mixed-precision form) everywhere else.  Errors are in units of each weight
   function's local scale (a power law in |x|, |y| fitted to the labels). */
struct kqed_surrogate_opts {
  size_t samples;   /* training samples, |x|, |y| log-uniform on the grid, cb uniform */
  size_t heldout;   /* held-out samples that set the per-cell error bounds */
  int batch;        /* samples per step, a multiple of 128 */
  int epochs;       /* passes over the training samples */
  double lr;        /* peak Adam learning rate (warm-up, cosine decay) */
  uint64_t seed;
  double tau;       /* initial acceptance bound */
};
struct kqed_surrogate_report {
  double loss_final;              /* mean-square training loss, last steps */
  double heldout_rms, heldout_max;      /* trained network, held-out samples */
  double untrained_rms, untrained_max;  /* the same network before training */
  double train_seconds;           /* wall time of the training steps */
  double steps;
  double cells_accepted;          /* fraction of cells whose bound is <= tau */
  double gemm_tflops;             /* tensor-core product rate during training */
  double seconds_total;           /* labels, training and bounds */
};
/* opts NULL: 1e7 samples, 1e6 held out, batch 8192, 4 epochs, lr 2e-3, tau 1e-3 */
int kqed_surrogate_train(const struct QED_kernel_temps *t, const struct kqed_surrogate_opts *opts,
                         struct kqed_surrogate_report *report);
int kqed_surrogate_set_tolerance(const struct QED_kernel_temps *t, double tau);
/* pairs the network evaluated in lattice sums since the last call (the
   counter is then reset); synchronises the device */
int kqed_surrogate_served(const struct QED_kernel_temps *t, uint64_t *served);
/* fraction of the feature cells whose bound is <= tau */
int kqed_surrogate_cells(const struct QED_kernel_temps *t, double tau, double *accepted_fraction);
/* at post-swap invariants d_u[n][3] = (|x|, |y|, cb) (device): the network's
   weight functions d_wnet[n][39] (float) and, if d_winterp != NULL, the FP64
   interpolation's d_winterp[n][39]; synchronises `stream` */
int kqed_surrogate_weights(const struct QED_kernel_temps *t, size_t n, const double *d_u,
                           float *d_wnet, double *d_winterp, void *stream);
/* the trained parameters (kqed_mlp_param_count() floats) and target scaling
   (9 + 3 * 39 floats: ln-range lo[3], scale[3], unused[3], oa[39], ob[39],
   os[39]); either may be NULL */
int kqed_surrogate_export(const struct QED_kernel_temps *t, float *params, float *norm);
size_t kqed_mlp_param_count(void);
/* One forward and backward pass of the network through the GPU kernels, no
   update, host buffers (for checking gradients): params as exported,
   feat[n][3] network inputs, target[n][39]; y[n][39] outputs, grad[params]
   of the mean-square loss, *loss.  n a multiple of 128. */
int kqed_mlp_forward_backward(const float *params, size_t n, const float *feat,
                              const float *target, float *y, float *grad, double *loss);
/* The network through the fused evaluation kernel that serves the lattice
   sums (layers 2-4 on the tensor cores with activations kept in shared
   memory), host buffers: y[n][39] for feat[n][3]. */
int kqed_mlp_infer(const float *params, size_t n, const float *feat, float *y);

/* Diagnostics.  kqed_profile(1) starts recording CUDA events on the
   launching stream around every main launch (the record + assembly kernel
   pair of the lattice sums and of the batched L0) and around every Pi chunk
   copy of kqed_lattice_sum; kqed_profile_read returns the launches' summed
   duration and count, kqed_profile_read_copies the copies'; kqed_profile(0)
   stops and clears.  kqed_fp64_peak_gflops runs an FP64 FMA-chain probe on
   the current device and returns GFLOP/s.  No reference counterpart. */
void kqed_profile(int enable);

/* The BF16 tensor-core GEMM (tcgen05, FP32 accumulation in tensor memory)
   that trains and evaluates the learned surrogate, exposed for testing; no
   reference counterpart.  d_c[z][m][n] = sum_{k in split z} A(m, k) B(n, k),
   A(m, k) = d_a[m * sam + k * sak], B(n, k) = d_b[n * sbn + k * sbk] (bf16,
   device), d_c fp32 with row stride ldc; split z of `splits` covers a
   contiguous range of k.  Synchronises `stream`. */
int kqed_bf16_gemm(const void *d_a, long long sam, long long sak, const void *d_b, long long sbn,
                   long long sbk, int M, int N, int K, int splits, float *d_c, long long ldc,
                   void *stream);
int kqed_profile_read(double *total_ms, uint64_t *launches);
int kqed_profile_read_copies(double *total_ms, uint64_t *copies);
int kqed_fp64_peak_gflops(double *gflops);
/* the same FMA-chain probe on the FP32 pipe (GFLOP/s) */
int kqed_fp32_peak_gflops(double *gflops);

#ifdef __cplusplus
}
#endif

#endif
