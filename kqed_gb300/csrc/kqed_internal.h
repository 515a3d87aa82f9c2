/*
 * Internal interface between the host layer (kqed_host.cpp) and the CUDA
 * kernels (kqed_fp64.cu).  Not installed; the public ABI is include/kqed.h.
 */
#ifndef KQED_INTERNAL_H
#define KQED_INTERNAL_H

#include <cuda_runtime.h>
#include <stddef.h>

#include <atomic>
#include <stdint.h>

struct QED_kernel_temps;

namespace kqed {

/* Weight-function tables, in the reference's FFidx order
   (src/HEADERS/KQED.h:50-53). */
enum {
  QG0, QG1, QG2, QG3, QL4, QL2, dxQG0, dxQG1, dxQG2, dxQG3, dxQL4, dxQL2, d2xQG2, d2xQG3,
  NFFA = 14
};

/* Slot of each table inside one 28-double node row.  Slots 0..7 are read by
   interpolation pass 1 (QG0,QL2,QL4,QG1 with their x-derivative partners),
   slots 8..13 by pass 2 (the QG2 and QG3 chains). */
static const int kSlotOfTable[NFFA] = {
    /*QG0*/ 0, /*QG1*/ 6, /*QG2*/ 8, /*QG3*/ 11, /*QL4*/ 4, /*QL2*/ 2,
    /*dxQG0*/ 1, /*dxQG1*/ 7, /*dxQG2*/ 9, /*dxQG3*/ 12, /*dxQL4*/ 5, /*dxQL2*/ 3,
    /*d2xQG2*/ 10, /*d2xQG3*/ 13};

/* number of leading zero Chebyshev coefficients a table carries: the "mm"
   shift of the reference's y-power scaling, src/LIBFILES/getff-new.c:126-128 */
static const int kShiftOfTable[NFFA] = {0, 0, 1, 0, 1, 2, 0, 0, 1, 0, 1, 2, 1, 0};

constexpr int kRow = 28;     /* doubles per (node, U-index) row: 14 tables x (value, y-derivative) */
constexpr int kNKMax = 64;   /* max Chebyshev length incl. the shift (nfx + 2) */
constexpr int kRec = 88;     /* doubles in the per-pair record between the two kernels */
constexpr int kTile = 64;    /* lattice sites per partial sum (unit = one x, kTile sites) */

/* Device-resident tables.  `node` holds, for every grid node (ix, iy) and
   Chebyshev index K (0..NK-1, U_K), the y-power-scaled coefficient of every
   table and its y-derivative, precomputed once at load time:
     node[((ix*nstpy + iy)*NK + K)*kRow + 2*slot + {0,1}]
   This is the value/derivative pair the reference recomputes inside every
   call (getff2, src/LIBFILES/getff-new.c:103-152); entries beyond a node's
   length are zero. */
struct DevTables {
  const double *XX, *YY; /* grids */
  const double *TX;      /* [23][ny_tay] TAYLORX */
  const double *TY;      /* [14][nx_tay] TAYLORY */
  const double *node;
  const float *node32;   /* the same table rounded to float (mixed-precision form) */
  const float2 *nodedf;  /* the same table as (hi, lo) floats (the FP64 form's double-float
                            Chebyshev sums in pair batches) */
  const int *nfx;
  int nstpx, nstpy, ny_tay, nx_tay, NK;
  double ystp;
};

/* Warp schedule of one STV -> 384 linear map: rows sorted by length and dealt
   to (round, lane) so the 32 lanes of a round do equal work. */
constexpr int kMapRounds = 12;
struct MapSched {
  int len[kMapRounds];      /* steps in each round */
  int off[kMapRounds];      /* first entry of each round (entries are [step][lane]) */
  int total;                /* entries in total (multiple of 32) */
};

/* The round lengths the two constant maps give (the float assembly unrolls
   its rounds with them; the host checks its schedules against them) */
__host__ __device__ constexpr int map_round_len(bool gen, int r)
{
  return gen ? (r == 0 ? 14 : r < 3 ? 13 : r == 3 ? 8 : r == 4 ? 7 : r < 8 ? 6 : r == 8 ? 4 : r < 11 ? 3 : 2)
             : (r < 3 ? 12 : r < 5 ? 8 : r < 7 ? 6 : r == 7 ? 5 : r == 8 ? 4 : r < 11 ? 3 : 2);
}

struct DevMaps {
  const uint16_t *ent_gen, *ent_zero;   /* col | code<<8 */
  const uint16_t *row_gen, *row_zero;   /* [round*32 + lane] -> output row */
  MapSched gen, zero;
};

/* Launch parameters chosen by the host (and the autotuner). */
struct LaunchCfg {
  int warps_per_block;   /* assembly kernels */
  int blocks;            /* assembly grid (0: occupancy-derived persistent grid) */
  double near_ratio;     /* mixed form: FP64 assembly when |x-y| < max(|x|,|y|)/near_ratio */
  double origin_radius;  /* mixed form: FP64 assembly when max(|x|,|y|) < origin_radius */
  int chnr32;            /* mixed form: chain rule in float for the float-assembled pairs
                            (off by default: +3.5% speed, per-pair mean error 3.2e-7
                            instead of 2.3e-7 on 1e7 random L3 pairs) */
};

/* Batched L0: out[i][384] for the pairs (x[i], y[i]). */
struct L0Args {
  const double *x, *y;  /* [n][4] */
  size_t n;
  double *out;          /* [n][384] */
  uint8_t *status;      /* [n] or NULL */
  double *rec;          /* record scratch [rec_cap][kRec] */
  uint8_t *code;        /* [rec_cap] */
  size_t rec_cap;       /* pairs per record kernel launch */
};

/* One fused lattice sum (or, in a batch, one job of it).  The record
   scratch fields are those of the launch (a batch uses the first
   descriptor's); u_begin is the job's first unit in the batch's unit list. */
struct LatticeArgs {
  const double *x;      /* [nx][4] */
  const double *y;      /* [ny][4] */
  size_t nx, ny;
  const double *pi;     /* [nx][ny][384], or NULL: generated (pi_seed, pi_stream, k0) */
  const double *Ky;     /* [ny][384] per-site additive kernel terms or NULL */
  const double *Bx;     /* [nx][384] per-x additive kernel terms or NULL */
  double *partial;      /* [nx][tiles][2]  (sum, compensation) */
  int tiles;            /* site tiles per x: ceil(ny / kTile) */
  const double *col;    /* per-x column tables [nx][nstpy][NK][kRow] or NULL */
  const float2 *Ky2, *Bx2;   /* Ky, Bx as float (hi, lo) pairs, for the mixed form */
  const float *col32;        /* column tables in float, for the mixed form */
  const float2 *coldf;       /* the FP64 column tables as (hi, lo) floats, for the FP64 form's
                                double-float Chebyshev sums, or NULL */
  double *rec;          /* record scratch [rec_cap][kRec] */
  uint8_t *code;        /* [rec_cap] */
  size_t rec_cap;       /* pairs per record kernel launch (a multiple of kTile) */
  double *env;          /* [rec_cap] Pi envelope per record (generated Pi) */
  uint32_t *list;       /* [rec_cap] mixed form: records left by the lean float pass */
  unsigned *count;      /* entries in list */
  uint64_t pi_seed;     /* generated Pi: Philox key */
  uint32_t pi_stream;   /* generated Pi: fourth counter word */
  size_t k0;            /* generated Pi: global index of x[0] */
  size_t n0;            /* generated Pi: global index of y[0] */
  size_t u_begin;       /* batch: first unit of this job */
  int zero_x_vanishes;  /* L2 / L3: at x = 0 every term cancels identically
                           (L2(0, y) = L0(0, y) - L0(0, y) - L0(0, 0)), so such pairs
                           contribute exactly zero and are skipped */
};

/* The learned weight-function surrogate as the lattice kernels see it (a
   device struct, filled by kqed_mlp.cu).  Features of a generic pair are its
   post-swap invariants u = (ln|x|, ln|y|, cb) mapped to [-1, 1]^3; the
   network predicts the 39 interpolated weight functions of interp_generic
   scaled by a power law, W_i = out_i * os_i * |x|^oa_i * |y|^ob_i. */
constexpr int kSurOut = 39;
constexpr int kSurOutPad = 48;   /* output layer width on the tensor cores */
struct SurDev {
  const float *cell;      /* [2][nb0][nb1][nb2] error bound of the network per feature cell:
                             the 37 weight functions of every pair, then all 39 (swapped
                             pairs also use the two y-derivative differences) */
  int nb[3];
  float lo[3], sc[3];     /* f_j = (u_j - lo_j) * sc_j - 1 */
  float tau;              /* a pair uses the network when its cell's bound <= tau */
  float oa[kSurOut], ob[kSurOut], os[kSurOut];
  float4 *feat;           /* [cap] features of the selected pairs, in selection order */
  uint32_t *elist;        /* [cap] record index of each selected pair */
  unsigned *ecount;       /* selected pairs */
  unsigned long long *etotal;   /* selected pairs summed over chunks (read by the host) */
  const float *Y;         /* [cap][kSurOutPad] network outputs in selection order */
};
/* host side of a lattice launch with the surrogate: d = the device struct;
   run(state, rows, stream) evaluates the network on the first *ecount of at
   most `rows` selected pairs (features -> Y) */
struct SurHook {
  const SurDev *d;
  unsigned *ecount;       /* the device counter of d (reset before each chunk) */
  cudaError_t (*run)(void *state, size_t rows, cudaStream_t s);
  void *state;
};
cudaError_t launch_lattice_surrogate(const DevTables &T, const DevMaps &M, const LatticeArgs &a,
                                     const LaunchCfg &cfg, const SurHook &hook, cudaStream_t s);
/* labels: W[i][39] = the FP64 interpolation at post-swap invariants
   u[i] = (|x|, |y|, cb), zero outside the grid */
cudaError_t launch_weight_labels(const DevTables &T, const double *u, size_t n, double *W,
                                 cudaStream_t s);
/* the surrogate attached to a device context (kqed_mlp.cu): the lattice
   launch hook for `cap` records per chunk, whether one exists, and its
   release when the context is freed */
int surrogate_hook(const void *ctx, size_t cap, SurHook *hook);
bool surrogate_ready(const void *ctx);
void surrogate_forget(const void *ctx);

int upload_map_constants();
cudaError_t launch_l0_fp64(const DevTables &T, const DevMaps &M, const L0Args &a,
                           const LaunchCfg &cfg, cudaStream_t s);
cudaError_t launch_lattice_fp64(const DevTables &T, const DevMaps &M, const LatticeArgs &a,
                                const LaunchCfg &cfg, cudaStream_t s);
/* a batch of lattices: d_jobs [njobs] on the device (u_begin ascending from
   0), `a` carries the record scratch; units = total units of all jobs */
cudaError_t launch_lattice_batch(const DevTables &T, const DevMaps &M, const LatticeArgs &a,
                                 const LatticeArgs *d_jobs, int njobs, size_t units,
                                 const LaunchCfg &cfg, cudaStream_t s, bool mixed);
cudaError_t launch_build_columns(const DevTables &T, const double *xs, size_t nx, double *col,
                                 cudaStream_t s);
cudaError_t launch_build_columns32(const DevTables &T, const double *xs, size_t nx, float *col,
                                   cudaStream_t s);
cudaError_t launch_l0_mixed(const DevTables &T, const DevMaps &M, const L0Args &a,
                            const LaunchCfg &cfg, cudaStream_t s);
cudaError_t launch_lattice_mixed(const DevTables &T, const DevMaps &M, const LatticeArgs &a,
                                 const LaunchCfg &cfg, cudaStream_t s);
cudaError_t launch_to_float2(const double *in, float2 *out, size_t n, cudaStream_t s);
cudaError_t launch_pi_synth(const double *xs, size_t nx, const double *ys, size_t ny, uint64_t seed,
                            uint32_t stream, size_t k0, size_t n0, double *pi, cudaStream_t s);
cudaError_t launch_stats(const double *A, const double *B, size_t m, double floor_abs, double *acc,
                         cudaStream_t s);
cudaError_t launch_reduce_partials(const double *partial, size_t nx, int tiles, double *sums,
                                   cudaStream_t s);
cudaError_t launch_axpy(double *y, const double *x, double a, size_t n, cudaStream_t s);
cudaError_t launch_scale(double *y, double a, size_t n, cudaStream_t s);
cudaError_t launch_mulam_axpy(double *y, const double *x, double a, size_t npairs,
                              cudaStream_t s);
cudaError_t launch_fill_pairs(const double *src, size_t n, int mode, double *dst,
                              cudaStream_t s);
size_t smem_bytes_l0(int warps_per_block);
cudaError_t probe_fp64_peak(double *gflops);
cudaError_t probe_fp32_peak(double *gflops);
extern std::atomic<uint64_t> g_launches;

/* device handles of an initialised struct QED_kernel_temps (0 on success) */
int ctx_handles(const struct QED_kernel_temps *t, DevTables *T, DevMaps *M, LaunchCfg *cfg);
/* record an error message for kqed_last_error(); returns 1 */
int set_error(const char *msg);
/* L0 over n device pairs, dout[n][384], in the given form (KQED_FP64 or
   KQED_FP32_MIXED), enqueued on s */
int l0_pairs(const struct QED_kernel_temps *t, const double *dx, const double *dy, size_t n,
             double *dout, int precision, cudaStream_t s);
/* the calling thread's device scratch (slot 0 or 1) of n doubles for this
   context, grown on demand; NULL on failure */
double *stage_scratch(const struct QED_kernel_temps *t, int slot, size_t n);
/* the calling thread's staging stream for this context */
cudaStream_t stage_stream(const struct QED_kernel_temps *t);
/* the device address of [p, p + bytes) when the range lies wholly inside
   one allocation of kqed_pinned_alloc (page-locked, device-mapped), which
   kernels may then read or write in place; NULL otherwise */
void *pinned_device(const void *p, size_t bytes);

} // namespace kqed

#endif
