/*
 * kqed_lattice_sum_noalloc: the fused lattice sum without any device memory
 * allocation.
 *
 * Some callers of this library cannot allocate GPU memory at the moment they
 * need the lattice sum: lattice QCD codes that hand the whole device to their
 * own memory pool at start-up and forbid foreign allocations, and tight loops
 * in which cudaMalloc/cudaFree would synchronise the device and stall the
 * caller's other streams.  kqed_lattice_sum_dev obtains its scratch (partial
 * sums per tile, the per-site and per-x kernel terms of L1..L3) with
 * cudaMalloc on first use; this entry point takes it from a fixed array
 * compiled into the library instead:
 *
 *   - the scratch is a file-scope static __device__ array of
 *     kNoallocDoubles doubles (16 MiB); every GPU that loads the library
 *     holds it until the process exits;
 *   - host code never uses the array's name as a device address (on the host
 *     it is only a stand-in symbol): the device address is obtained with
 *     cudaGetSymbolAddress, with the device current, on the first call made
 *     in each CUDA context -- once per device, and again after a
 *     cudaDeviceReset has replaced the device's primary context (the cached
 *     address is keyed by the context's unique id).  Make that first call
 *     before any stream capture;
 *   - problems whose scratch does not fit are rejected with an error that
 *     states the need and the limit; nothing is allocated, here or in any
 *     library routine this function calls.  The per-pair records passed
 *     between the record and assembly kernels take whatever room is left
 *     (at least one tile of kTile pairs); with less room the same kernels
 *     run in more, smaller launches;
 *   - all calls share the one array and it keeps the last call's contents.
 *     Everything a call reads from it is first written by the same call (the
 *     zero vectors are cleared by a kernel, partial sums and kernel terms are
 *     fully overwritten), but calls that overlap on the GPU -- on different
 *     streams, or from different host threads -- race on the array and must
 *     be serialised by the caller.
 *
 * Results agree with kqed_lattice_sum_dev's to about 1e-12 relative, not bit
 * for bit: the reduction order is the same, but without room for the per-x
 * column tables the record kernel interpolates from the node table (the
 * path of the pair batches), and the contraction splits the FP64 per-site
 * and per-x terms into (hi, lo) floats in the kernel instead of reading a
 * prebuilt split.
 */
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/kqed.h"
#include "kqed_internal.h"

namespace {

constexpr size_t kNoallocDoubles = (size_t)2 << 20; /* 2,097,152 doubles = 16 MiB */

static __device__ __align__(256) double g_noalloc_scratch[kNoallocDoubles];

constexpr int kMaxDevices = 64;
struct ScratchSlot {
  unsigned long long ctx_id; /* 0: not looked up yet */
  double *addr;
};
ScratchSlot g_scratch[kMaxDevices] = {};
std::mutex g_scratch_mu;

typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);

/* unique id of the calling thread's current CUDA context (0 if none); the
   driver functions are reached through the runtime, so the library does not
   link the driver library itself */
unsigned long long current_ctx_id()
{
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  if (!get_current || !get_id) return 0;
  void *ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

/* device address of the static scratch in the current context (looked up
   with cudaGetSymbolAddress on the first call in each context) */
int scratch_on_current_device(double **out)
{
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return kqed::set_error("kqed_lattice_sum_noalloc: no usable current CUDA device");
  unsigned long long id = current_ctx_id();
  if (id == 0) {   /* no context yet on this thread: make the device's primary one current */
    if (cudaSetDevice(dev) != cudaSuccess)
      return kqed::set_error("kqed_lattice_sum_noalloc: cannot make the device current");
    id = current_ctx_id();
  }
  std::lock_guard<std::mutex> g(g_scratch_mu);
  ScratchSlot &sl = g_scratch[dev];
  if (!sl.addr || id == 0 || sl.ctx_id != id) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      char msg[256];
      snprintf(msg, sizeof(msg), "kqed_lattice_sum_noalloc: cudaGetSymbolAddress failed: %s",
               cudaGetErrorString(e));
      return kqed::set_error(msg);
    }
    sl.addr = static_cast<double *>(p);
    sl.ctx_id = id;
  }
  *out = sl.addr;
  return 0;
}

struct Recs {
  double *rec;
  uint8_t *code;
  size_t cap;
};

int l0(const kqed::DevTables &T, const kqed::DevMaps &M, const kqed::LaunchCfg &cfg,
       const double *dx, const double *dy, size_t n, double *out, const Recs &R, cudaStream_t s)
{
  kqed::L0Args a{dx, dy, n, out, nullptr, R.rec, R.code, R.cap};
  return kqed::launch_l0_fp64(T, M, a, cfg, s) != cudaSuccess;
}

} // namespace

extern "C" int kqed_lattice_sum_noalloc(const struct QED_kernel_temps *t, int variant, size_t nx,
                                        const double *d_x, size_t ny, const double *d_y,
                                        const double *d_pi, double *d_sums, void *stream)
{
  kqed::DevTables T;
  kqed::DevMaps M;
  kqed::LaunchCfg cfg;
  if (kqed::ctx_handles(t, &T, &M, &cfg)) return kqed::set_error("tables not initialised");
  if (variant < 0 || variant > 3) return kqed::set_error("variant not in 0..3");
  if (nx == 0) return 0;
  if (!d_sums) return kqed::set_error("null buffer");
  if (ny == 0) {   /* an empty lattice sums to zero (its site and Pi pointers may be NULL) */
    if (cudaMemsetAsync(d_sums, 0, nx * sizeof(double), static_cast<cudaStream_t>(stream)) !=
        cudaSuccess)
      return kqed::set_error("kqed_lattice_sum_noalloc: memset failed");
    return 0;
  }
  if (!d_x || !d_y || !d_pi) return kqed::set_error("null buffer");
  if (nx > kNoallocDoubles || ny > kNoallocDoubles) {
    /* bounded first, so that the scratch arithmetic below cannot wrap */
    char msg[256];
    snprintf(msg, sizeof(msg),
             "kqed_lattice_sum_noalloc: %zu x points x %zu sites exceed the static limit of "
             "%zu doubles of scratch (16 MiB). Use kqed_lattice_sum_dev.", nx, ny,
             kNoallocDoubles);
    return kqed::set_error(msg);
  }
  const size_t tiles = (ny + kqed::kTile - 1) / kqed::kTile;
  const size_t n_partial = nx * (tiles ? tiles : 1) * 2;
  const size_t n_terms = variant ? ny * 384 + ny * 4 + nx * 384 * 2 + nx * 4 : 0;
  /* one tile of records at least: kTile pairs of kRec doubles + their codes */
  const size_t rec_tile = (size_t)kqed::kTile * kqed::kRec + kqed::kTile / 8;
  const size_t need = n_partial + n_terms + rec_tile;
  if (need > kNoallocDoubles) {
    char msg[320];
    snprintf(msg, sizeof(msg),
             "kqed_lattice_sum_noalloc: %zu x points x %zu sites (L%d) need %zu doubles of "
             "scratch; the static limit is %zu doubles (16 MiB). Use kqed_lattice_sum_dev.",
             nx, ny, variant, need, kNoallocDoubles);
    return kqed::set_error(msg);
  }
  double *S = nullptr;
  if (scratch_on_current_device(&S)) return 1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double *partial = S;
  /* records in the room after the partial sums and kernel terms */
  Recs RC;
  {
    const size_t room = kNoallocDoubles - n_partial - n_terms;
    size_t cap = room * 8 / (8 * (size_t)kqed::kRec + 1);
    cap = cap / kqed::kTile * kqed::kTile;
    RC.rec = S + n_partial + n_terms;
    RC.code = reinterpret_cast<uint8_t *>(RC.rec + cap * kqed::kRec);
    RC.cap = cap;
  }
  double *Ky = nullptr, *Bx = nullptr;
  if (variant) {
    Ky = partial + n_partial;
    double *zy = Ky + ny * 384;
    Bx = zy + ny * 4;
    double *bt = Bx + nx * 384;
    double *zx = bt + nx * 384;
    int bad = kqed::launch_fill_pairs(nullptr, ny, 0, zy, s) != cudaSuccess ||
              kqed::launch_fill_pairs(nullptr, nx, 0, zx, s) != cudaSuccess;
    /* the per-site and per-x terms of QED_kernel_L1..L3, src/LIBFILES/kernels.c:117-177 */
    switch (variant) {
    case 1:
      bad = bad || l0(T, M, cfg, d_y, d_y, ny, Ky, RC, s) || l0(T, M, cfg, d_x, d_x, nx, Bx, RC, s) ||
            kqed::launch_scale(Ky, -0.5, ny * 384, s) != cudaSuccess ||
            kqed::launch_scale(Bx, -0.5, nx * 384, s) != cudaSuccess;
      break;
    case 2:
      bad = bad || l0(T, M, cfg, zy, d_y, ny, Ky, RC, s) || l0(T, M, cfg, d_x, zx, nx, Bx, RC, s) ||
            kqed::launch_scale(Ky, -1.0, ny * 384, s) != cudaSuccess ||
            kqed::launch_scale(Bx, -1.0, nx * 384, s) != cudaSuccess;
      break;
    default:
      bad = bad || l0(T, M, cfg, zy, d_y, ny, Ky, RC, s) || l0(T, M, cfg, d_x, d_x, nx, Bx, RC, s) ||
            l0(T, M, cfg, zx, d_x, nx, bt, RC, s) ||
            kqed::launch_scale(Ky, -1.0, ny * 384, s) != cudaSuccess ||
            kqed::launch_scale(Bx, -1.0, nx * 384, s) != cudaSuccess ||
            kqed::launch_axpy(Bx, bt, 1.0, nx * 384, s) != cudaSuccess;
      break;
    }
    if (bad) return kqed::set_error("kqed_lattice_sum_noalloc: kernel-term launch failed");
  }
  kqed::LatticeArgs a{};
  a.x = d_x;
  a.y = d_y;
  a.nx = nx;
  a.ny = ny;
  a.pi = d_pi;
  a.Ky = Ky;
  a.Bx = Bx;
  a.partial = partial;
  a.tiles = (int)tiles;
  a.rec = RC.rec;
  a.code = RC.code;
  a.rec_cap = RC.cap;
  a.zero_x_vanishes = variant >= 2;
  if (kqed::launch_lattice_fp64(T, M, a, cfg, s) != cudaSuccess ||
      kqed::launch_reduce_partials(partial, nx, (int)tiles, d_sums, s) != cudaSuccess)
    return kqed::set_error("kqed_lattice_sum_noalloc: lattice kernel launch failed");
  return 0;
}
