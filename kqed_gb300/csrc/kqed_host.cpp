/*
 * Host layer of libkqed_gb300.so: the reference-compatible C API
 * (initialise / free_QED_temps / QED_kernel_L0..L3) and the batched and fused
 * entry points, over the sm_103a kernels in kqed_fp64.cu.
 *
 * Tables are read from the reference's own files and formats
 * (src/LIBFILES/io.c:42-289), checksummed the same way
 * (src/UTILS/crc32c.c:160-172), and precomputed once into the device layout
 * described in kqed_internal.h.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/kqed.h"
#include "kqed_crc32c.h"
#include "kqed_internal.h"
#include "kqed_stv_map.h"

#ifndef KQED_DEFAULT_LIB_PATH
#define KQED_DEFAULT_LIB_PATH "."
#endif

using namespace kqed;

/* ------------------------------------------------------------- errors */

static thread_local std::string tl_err;

static int fail(const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  tl_err = buf;
  return 1;
}

#define CUDA_OK(call)                                                                      \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return fail("%s: %s", #call, cudaGetErrorString(e_));           \
  } while (0)

extern "C" const char *kqed_last_error(void) { return tl_err.c_str(); }
extern "C" uint64_t kqed_launch_count(void) { return kqed::g_launches; }

/* ------------------------------------------------------ kernel timing */

/* CUDA events recorded on the launching stream around every main launch
   (the lattice and batched-L0 kernel pairs; kind 0) and around the chunk
   copies of the host entry points (kind 1) while enabled */
namespace {
struct TimedLaunch { cudaEvent_t a, b; int kind; };
std::mutex g_prof_mu;
std::vector<TimedLaunch> g_prof;
std::atomic<int> g_prof_on{0};
} // namespace

static void prof_begin(cudaStream_t s, TimedLaunch &tl, int kind = 0)
{
  tl.a = tl.b = nullptr;
  tl.kind = kind;
  if (!g_prof_on) return;
  cudaEventCreate(&tl.a);
  cudaEventCreate(&tl.b);
  cudaEventRecord(tl.a, s);
}

static void prof_end(cudaStream_t s, TimedLaunch &tl)
{
  if (!tl.a) return;
  cudaEventRecord(tl.b, s);
  std::lock_guard<std::mutex> g(g_prof_mu);
  g_prof.push_back(tl);
}

extern "C" void kqed_profile(int enable)
{
  std::lock_guard<std::mutex> g(g_prof_mu);
  for (auto &t : g_prof) { cudaEventDestroy(t.a); cudaEventDestroy(t.b); }
  g_prof.clear();
  g_prof_on = enable ? 1 : 0;
}

static int profile_sum(int kind, double *total_ms, uint64_t *count)
{
  std::lock_guard<std::mutex> g(g_prof_mu);
  double tot = 0;
  uint64_t n = 0;
  for (auto &t : g_prof) {
    if (t.kind != kind) continue;
    if (cudaEventSynchronize(t.b) != cudaSuccess) return fail("event sync failed");
    float ms = 0;
    cudaEventElapsedTime(&ms, t.a, t.b);
    tot += ms;
    n++;
  }
  *total_ms = tot;
  *count = n;
  return 0;
}

extern "C" int kqed_profile_read(double *total_ms, uint64_t *launches)
{
  return profile_sum(0, total_ms, launches);
}

extern "C" int kqed_profile_read_copies(double *total_ms, uint64_t *copies)
{
  return profile_sum(1, total_ms, copies);
}

extern "C" int kqed_fp64_peak_gflops(double *gflops)
{
  CUDA_OK(probe_fp64_peak(gflops));
  return 0;
}

extern "C" int kqed_fp32_peak_gflops(double *gflops)
{
  CUDA_OK(probe_fp32_peak(gflops));
  return 0;
}


/* ---------------------------------------------------------- context */

namespace {

struct Scratch {
  double *buf = nullptr;
  size_t cap = 0; /* doubles */
  double *get(size_t n)
  {
    if (n > cap) {
      /* work queued on any stream may still use the old buffer */
      if (buf) {
        cudaDeviceSynchronize();
        cudaFree(buf);
      }
      buf = nullptr;
      cap = 0;
      if (cudaMalloc(&buf, n * sizeof(double)) != cudaSuccess) return nullptr;
      cap = n;
    }
    return buf;
  }
  void release()
  {
    if (buf) cudaFree(buf);
    buf = nullptr;
    cap = 0;
  }
};

std::atomic<uint64_t> g_ctx_ids{0};

struct Ctx {
  /* unique for the life of the process: a later context may reuse a freed
     one's address (and sit on another device) */
  uint64_t id = ++g_ctx_ids;
  int device = 0;
  DevTables T{};
  DevMaps M{};
  LaunchCfg cfg{4, 0, 4.0, 0.35, 0};
  std::vector<void *> allocs;
};

/* per-thread staging for the per-pair legacy calls and batched host calls */
struct ThreadStage {
  uint64_t owner = 0;       /* Ctx::id of the context the streams and buffers serve */
  cudaStream_t stream = nullptr, copy_stream = nullptr;
  cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr};
  double *h_pin = nullptr;   /* 8 + 384 doubles */
  Scratch d_io, d_tmp, d_aux, d_aux2, d_col, d_col32, d_rec, d_rec2, d_sa, d_sb, d_cmp, d_cmp_io;
  ~ThreadStage() { reset(); }
  void reset()
  {
    if (stream) cudaStreamDestroy(stream);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    for (int i = 0; i < 2; i++) {
      if (ev_copied[i]) cudaEventDestroy(ev_copied[i]);
      if (ev_free[i]) cudaEventDestroy(ev_free[i]);
      ev_copied[i] = ev_free[i] = nullptr;
    }
    copy_stream = nullptr;
    if (h_pin) cudaFreeHost(h_pin);
    d_io.release(); d_tmp.release(); d_aux.release(); d_aux2.release(); d_col.release(); d_col32.release();
    d_rec.release(); d_rec2.release(); d_sa.release(); d_sb.release(); d_cmp.release(); d_cmp_io.release();
    stream = nullptr;
    h_pin = nullptr;
    owner = 0;
  }
};

thread_local ThreadStage tl_stage;

static ThreadStage &stage_for(Ctx *c)
{
  ThreadStage &st = tl_stage;
  if (st.owner != c->id) {
    st.reset();
    st.owner = c->id;
  }
  return st;
}

/* Per-pair records between the record and assembly kernels: room for up to
   kRecPairs pairs (712 bytes each) per launch pair, a multiple of kTile. */
constexpr size_t kRecPairs = (size_t)1 << 20;

Ctx *ctx_of(const struct QED_kernel_temps *t)
{
  if (!t || !t->Grid.PC) return nullptr;
  return static_cast<Ctx *>(t->Grid.PC->Fm);
}

} // namespace

/* ------------------------------------------------------------- loading */

static int rd(void *p, size_t sz, size_t n, FILE *f) { return fread(p, sz, n, f) != n; }

static std::string lib_path()
{
  const char *e = getenv("KQED_LIB_PATH");
  return e && *e ? std::string(e) : std::string(KQED_DEFAULT_LIB_PATH);
}

/* read_ff, src/LIBFILES/io.c:42-176, filling the reference's Grid fields */
static int load_ff(const std::string &lib, struct Grid_coeffs *G)
{
  const std::string path = lib + "/PRECOMP/FFxy_single_cksum.bin";
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return fail("Cannot find %s", path.c_str());
  int magic = 0, n = 0;
  uint32_t ck[2], a, b;
  std::string why;
  if (rd(&magic, 4, 1, f) || magic != 816968) { why = "missing magic number"; goto bad; }
  if (rd(&n, 4, 1, f) || n < 2 || n > 100000) { why = "bad nstpx"; goto bad; }
  G->nstpx = n;
  G->XX = (double *)malloc(sizeof(double) * n);
  if (rd(G->XX, 8, n, f) || rd(ck, 4, 2, f)) { why = "truncated XX"; goto bad; }
  a = b = 0;
  kqed_cksum_accum(&a, &b, 0, G->XX, sizeof(double) * n);
  if (a != ck[0] || b != ck[1]) { why = "XX checksum mismatch"; goto bad; }
  if (rd(&n, 4, 1, f) || n < 2 || n > 100000) { why = "bad nstpy"; goto bad; }
  G->nstpy = n;
  G->YY = (double *)malloc(sizeof(double) * n);
  if (rd(G->YY, 8, n, f) || rd(ck, 4, 2, f)) { why = "truncated YY"; goto bad; }
  a = b = 0;
  kqed_cksum_accum(&a, &b, 0, G->YY, sizeof(double) * n);
  if (a != ck[0] || b != ck[1]) { why = "YY checksum mismatch"; goto bad; }
  G->xstp = G->XX[1] - G->XX[0];
  G->ystp = G->YY[1] - G->YY[0];
  if (rd(&G->Nffa, 4, 1, f) || G->Nffa != NFFA) { why = "bad Nffa"; goto bad; }
  G->nfx = (int *)calloc(G->nstpx, sizeof(int));
  G->Ffm = (float ****)calloc(G->Nffa, sizeof(float ***));
  G->Ffp = (float ****)calloc(G->Nffa, sizeof(float ***));
  {
    uint32_t ma = 0, mb = 0, pa = 0, pb = 0, rank = 0;
    for (int ia = 0; ia < G->Nffa; ia++) {
      if (rd(&n, 4, 1, f) || n != G->nstpx) { why = "file is funny nstpx"; goto bad; }
      G->Ffm[ia] = (float ***)calloc(G->nstpx, sizeof(float **));
      G->Ffp[ia] = (float ***)calloc(G->nstpx, sizeof(float **));
      for (int ix = 0; ix < G->nstpx; ix++) {
        if (rd(&n, 4, 1, f) || n != G->nstpy) { why = "file is funny nstpy"; goto bad; }
        G->Ffm[ia][ix] = (float **)calloc(G->nstpy, sizeof(float *));
        G->Ffp[ia][ix] = (float **)calloc(G->nstpy, sizeof(float *));
        for (int iy = 0; iy < G->nstpy; iy++) {
          int nf = 0;
          if (rd(&nf, 4, 1, f) || nf < 1 || nf > kNKMax - 2) { why = "bad coefficient count"; goto bad; }
          if (G->nfx[ix] && G->nfx[ix] != nf) { why = "ragged coefficient count within an x node"; goto bad; }
          G->nfx[ix] = nf;
          float *fm = (float *)malloc(sizeof(float) * nf), *fp = (float *)malloc(sizeof(float) * nf);
          G->Ffm[ia][ix][iy] = fm;
          G->Ffp[ia][ix][iy] = fp;
          if (rd(fm, 4, nf, f)) { why = "truncated coefficients"; goto bad; }
          kqed_cksum_accum(&ma, &mb, rank, fm, sizeof(float) * nf);
          if (rd(fp, 4, nf, f)) { why = "truncated coefficients"; goto bad; }
          kqed_cksum_accum(&pa, &pb, rank, fp, sizeof(float) * nf);
          rank++;
        }
      }
    }
    uint32_t tail[4];
    if (rd(tail, 4, 4, f)) { why = "truncated checksums"; goto bad; }
    if (tail[0] != ma || tail[1] != mb || tail[2] != pa || tail[3] != pb) {
      why = "Computed and read ff checksums do not match";
      goto bad;
    }
  }
  fclose(f);
  return 0;
bad:
  fclose(f);
  return fail("|IO| %s: %s", path.c_str(), why.c_str());
}

/* read_TAYLORX / read_TAYLORY, src/LIBFILES/io.c:179-289 */
static int load_taylor(const std::string &lib, const char *name, int nrows, int ncols,
                       double ***rows_out, int *nrows_out, int *ncols_out)
{
  const std::string path = lib + "/PRECOMP/" + name;
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return fail("|IO| cannot open %s", path.c_str());
  int magic = 0, n = 0;
  uint32_t a = 0, b = 0, ck[2];
  double **rows = (double **)calloc(nrows, sizeof(double *));
  *rows_out = rows;
  *nrows_out = nrows;
  if (rd(&magic, 4, 1, f) || magic != 816968 || rd(&n, 4, 1, f) || n != nrows) goto bad;
  for (int i = 0; i < nrows; i++) {
    int m = 0;
    if (rd(&m, 4, 1, f) || m != ncols) goto bad;
    rows[i] = (double *)malloc(sizeof(double) * m);
    if (rd(rows[i], 8, m, f)) goto bad;
    kqed_cksum_accum(&a, &b, (uint32_t)i, rows[i], sizeof(double) * m);
  }
  if (rd(ck, 4, 2, f) || ck[0] != a || ck[1] != b) goto bad;
  *ncols_out = ncols;
  fclose(f);
  return 0;
bad:
  fclose(f);
  return fail("|IO| %s malformed or checksums do not match", path.c_str());
}

/* ------------------------------------------- table readers and writers */

/* read_ff / read_TAYLORX / read_TAYLORY, src/LIBFILES/io.c:42-289
   (src/HEADERS/io.h:4-11): fill the Grid fields from LIB_PATH/PRECOMP with
   checksum validation; 0 on success, 1 with a message on failure */
extern "C" int read_ff(struct Grid_coeffs *Grid)
{
  if (!Grid) return fail("null grid");
  if (load_ff(lib_path(), Grid)) {
    fprintf(stderr, "%s\n", tl_err.c_str());
    return 1;
  }
  return 0;
}

extern "C" int read_TAYLORX(struct Grid_coeffs *Grid)
{
  if (!Grid) return fail("null grid");
  if (load_taylor(lib_path(), "taylorx_cksum.bin", 23, 810, &Grid->TX, &Grid->NtayY, &Grid->NY_tay)) {
    fprintf(stderr, "%s\n", tl_err.c_str());
    return 1;
  }
  return 0;
}

extern "C" int read_TAYLORY(struct Grid_coeffs *Grid)
{
  if (!Grid) return fail("null grid");
  if (load_taylor(lib_path(), "taylory_cksum.bin", 14, 100, &Grid->TY, &Grid->NtayX, &Grid->NX_tay)) {
    fprintf(stderr, "%s\n", tl_err.c_str());
    return 1;
  }
  return 0;
}

/* the checksummed table writers of src/LIBFILES/io.c:292-412: the same
   layouts (magic 816968, counts, values, rank-rotated CRC32C pairs), the
   same relative paths under ./PRECOMP (write_ff to FFxy_single_cksum2.bin,
   so that the table in use is not overwritten) */
static bool wr(FILE *f, const void *p, size_t sz, size_t n) { return fwrite(p, sz, n, f) == n; }

extern "C" void write_ff(const struct Grid_coeffs *G)
{
  FILE *f = G ? fopen("./PRECOMP/FFxy_single_cksum2.bin", "wb") : nullptr;
  if (!f) {
    fprintf(stderr, "|IO| cannot write ./PRECOMP/FFxy_single_cksum2.bin\n");
    return;
  }
  const int magic = 816968;
  bool ok = wr(f, &magic, 4, 1);
  uint32_t ck[2];
  ck[0] = ck[1] = 0;
  kqed_cksum_accum(&ck[0], &ck[1], 0, G->XX, sizeof(double) * G->nstpx);
  ok = ok && wr(f, &G->nstpx, 4, 1) && wr(f, G->XX, 8, G->nstpx) && wr(f, ck, 4, 2);
  ck[0] = ck[1] = 0;
  kqed_cksum_accum(&ck[0], &ck[1], 0, G->YY, sizeof(double) * G->nstpy);
  ok = ok && wr(f, &G->nstpy, 4, 1) && wr(f, G->YY, 8, G->nstpy) && wr(f, ck, 4, 2);
  ok = ok && wr(f, &G->Nffa, 4, 1);
  uint32_t ma = 0, mb = 0, pa = 0, pb = 0, rank = 0;
  for (int ia = 0; ok && ia < G->Nffa; ia++) {
    ok = wr(f, &G->nstpx, 4, 1);
    for (int ix = 0; ok && ix < G->nstpx; ix++) {
      const int nf = G->nfx[ix];
      ok = wr(f, &G->nstpy, 4, 1);
      for (int iy = 0; ok && iy < G->nstpy; iy++, rank++) {
        const float *fm = G->Ffm[ia][ix][iy], *fp = G->Ffp[ia][ix][iy];
        ok = wr(f, &nf, 4, 1) && wr(f, fm, 4, nf) && wr(f, fp, 4, nf);
        kqed_cksum_accum(&ma, &mb, rank, fm, sizeof(float) * nf);
        kqed_cksum_accum(&pa, &pb, rank, fp, sizeof(float) * nf);
      }
    }
  }
  const uint32_t tail[4] = {ma, mb, pa, pb};
  ok = ok && wr(f, tail, 4, 4);
  if (fclose(f) != 0 || !ok) fprintf(stderr, "|IO| write of FFxy_single_cksum2.bin failed\n");
}

static void write_taylor(const char *path, const char *what, int nrows, int ncols,
                         double *const *rows)
{
  FILE *f = fopen(path, "wb");
  if (!f) {
    fprintf(stderr, "|IO| cannot write to file %s\n", what);
    return;
  }
  const int magic = 816968;
  bool ok = wr(f, &magic, 4, 1) && wr(f, &nrows, 4, 1);
  uint32_t a = 0, b = 0;
  for (int i = 0; ok && i < nrows; i++) {
    ok = wr(f, &ncols, 4, 1) && wr(f, rows[i], 8, ncols);
    kqed_cksum_accum(&a, &b, (uint32_t)i, rows[i], sizeof(double) * ncols);
  }
  ok = ok && wr(f, &a, 4, 1) && wr(f, &b, 4, 1);
  if (fclose(f) != 0 || !ok) fprintf(stderr, "|IO| write of %s failed\n", path);
}

extern "C" void write_TAYLORX(const struct Grid_coeffs *G)
{
  if (G) write_taylor("./PRECOMP/taylorx_cksum.bin", "TAYLORX", G->NtayY, G->NY_tay, G->TX);
}

extern "C" void write_TAYLORY(const struct Grid_coeffs *G)
{
  if (G) write_taylor("./PRECOMP/taylory_cksum.bin", "TAYLORY", G->NtayX, G->NX_tay, G->TY);
}

/* the reference's per-call y-power scaling (getff2, src/LIBFILES/getff-new.c:103-152),
   applied once per node; out arrays are indexed by Chebyshev index U_K */
static void scale_node(int nm, double y, int nf, const float *fm, const float *fp, double *fval,
                       double *fvalD)
{
  const double y1 = 1.0 / y;
  double yp = 1;
  int mshm = 2;
  switch (nm) {
  case QG2: case dxQG2: case d2xQG2: yp = y1; mshm = 3; break;
  case QL4: case dxQL4: yp = y; mshm = 1; break;
  case QL2: case dxQL2: yp = y1 * y1; mshm = 4; break;
  default: yp = 1.0; mshm = 2; break;
  }
  int mshp = 2 - mshm;
  const int mm = abs(mshp);
  double facm = y1 * y1 * yp, facp = yp;
  for (int j = 0; j < mm; j++) { facm *= y1; facp *= y; }
  mshm += mm; mshp += mm;
  for (int j = 0; j < nf; j++) {
    fvalD[mm + j] = y1 * mshp * facp * (double)fp[j] - y1 * mshm * facm * (double)fm[j];
    fval[mm + j] = facm * (double)fm[j] + facp * (double)fp[j];
    facm *= y1; facp *= y;
    mshm++; mshp++;
  }
}

static void *dev_upload(Ctx *c, const void *h, size_t bytes)
{
  void *d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) return nullptr;
  if (cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess) { cudaFree(d); return nullptr; }
  c->allocs.push_back(d);
  return d;
}

/* deal the rows of a sparse map to (round, lane) by length */
static int build_sched(const unsigned short *row, const unsigned char *col, const signed char *q4,
                       MapSched &S, std::vector<uint16_t> &ent, std::vector<uint16_t> &rows)
{
  std::vector<int> order(384);
  for (int i = 0; i < 384; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (row[a + 1] - row[a]) > (row[b + 1] - row[b]);
  });
  rows.assign(384, 0);
  ent.clear();
  int off = 0;
  for (int r = 0; r < kMapRounds; r++) {
    int len = 0;
    for (int l = 0; l < 32; l++) {
      const int i = order[r * 32 + l];
      len = std::max(len, (int)(row[i + 1] - row[i]));
      rows[r * 32 + l] = (uint16_t)i;
    }
    S.len[r] = len;
    S.off[r] = off;
    for (int s = 0; s < len; s++)
      for (int l = 0; l < 32; l++) {
        const int i = order[r * 32 + l];
        const int nz = row[i + 1] - row[i];
        uint16_t e = (uint16_t)200; /* padding: the zero slot, coefficient 1 */
        if (s < nz) {
          const int k = row[i] + s;
          /* codes 0..5 = coefficients 1, -1, 2, -2, 1/2, -1/2: the float
             assembly reads the product from a table at code * 256 + col, and
             in this order (the 1/2 terms use columns 0..7 only) the table
             spans 1288 floats */
          int code;
          switch (q4[k]) {
          case 4: code = 0; break;
          case -4: code = 1; break;
          case 8: code = 2; break;
          case -8: code = 3; break;
          case 2: code = 4; break;
          case -2: code = 5; break;
          default: return 1;
          }
          if (code >= 4 && col[k] >= 8) return 1;
          e = (uint16_t)(col[k] | (code << 8));
        }
        ent.push_back(e);
      }
    off += len * 32;
  }
  S.total = off;
  const bool gen = row == KQ_MAP_GEN_ROW;
  for (int r = 0; r < kMapRounds; r++)
    if (S.len[r] != map_round_len(gen, r)) return 1;
  return off > 3072 ? 1 : 0;
}

static int setup_device(struct Grid_coeffs *G, Ctx *c)
{
  CUDA_OK(cudaGetDevice(&c->device));
  if (upload_map_constants()) return fail("cannot upload Clenshaw constants");
  int nfmax = 0;
  for (int i = 0; i < G->nstpx; i++) nfmax = std::max(nfmax, G->nfx[i]);
  const int NK = nfmax + 2;
  if (NK > kNKMax) return fail("Chebyshev length %d exceeds %d", NK, kNKMax);
  /* node table */
  const size_t nrow = (size_t)G->nstpx * G->nstpy * NK;
  std::vector<double> node(nrow * kRow, 0.0);
  std::vector<double> fval(kNKMax + 2), fvalD(kNKMax + 2);
  for (int a = 0; a < NFFA; a++)
    for (int ix = 0; ix < G->nstpx; ix++)
      for (int iy = 0; iy < G->nstpy; iy++) {
        std::fill(fval.begin(), fval.end(), 0.0);
        std::fill(fvalD.begin(), fvalD.end(), 0.0);
        const int nf = G->nfx[ix];
        scale_node(a, G->YY[iy], nf, G->Ffm[a][ix][iy], G->Ffp[a][ix][iy], fval.data(), fvalD.data());
        const int len = nf + kShiftOfTable[a];
        double *base = node.data() + ((size_t)ix * G->nstpy + iy) * NK * kRow + 2 * kSlotOfTable[a];
        for (int K = 0; K < len; K++) {
          base[(size_t)K * kRow + 0] = fval[K];
          base[(size_t)K * kRow + 1] = fvalD[K];
        }
      }
  std::vector<double> tx(23 * (size_t)G->NY_tay), ty(14 * (size_t)G->NX_tay);
  for (int r = 0; r < 23; r++) memcpy(&tx[(size_t)r * G->NY_tay], G->TX[r], sizeof(double) * G->NY_tay);
  for (int r = 0; r < 14; r++) memcpy(&ty[(size_t)r * G->NX_tay], G->TY[r], sizeof(double) * G->NX_tay);
  DevTables &T = c->T;
  T.XX = (const double *)dev_upload(c, G->XX, sizeof(double) * G->nstpx);
  T.YY = (const double *)dev_upload(c, G->YY, sizeof(double) * G->nstpy);
  T.TX = (const double *)dev_upload(c, tx.data(), sizeof(double) * tx.size());
  T.TY = (const double *)dev_upload(c, ty.data(), sizeof(double) * ty.size());
  T.node = (const double *)dev_upload(c, node.data(), sizeof(double) * node.size());
  {
    std::vector<float> node32(node.size());
    for (size_t i = 0; i < node.size(); i++) node32[i] = (float)node[i];
    T.node32 = (const float *)dev_upload(c, node32.data(), sizeof(float) * node32.size());
  }
  {
    std::vector<float2> nodedf(node.size());
    for (size_t i = 0; i < node.size(); i++) {
      const float hi = (float)node[i];
      nodedf[i] = make_float2(hi, (float)(node[i] - (double)hi));
    }
    T.nodedf = (const float2 *)dev_upload(c, nodedf.data(), sizeof(float2) * nodedf.size());
  }
  T.nfx = (const int *)dev_upload(c, G->nfx, sizeof(int) * G->nstpx);
  if (!T.XX || !T.YY || !T.TX || !T.TY || !T.node || !T.node32 || !T.nodedf || !T.nfx)
    return fail("device table upload failed");
  T.nstpx = G->nstpx; T.nstpy = G->nstpy; T.ny_tay = G->NY_tay; T.nx_tay = G->NX_tay; T.NK = NK;
  T.ystp = G->ystp;
  /* map schedules */
  std::vector<uint16_t> eg, rg, ez, rz;
  if (build_sched(KQ_MAP_GEN_ROW, KQ_MAP_GEN_COL, KQ_MAP_GEN_Q4, c->M.gen, eg, rg) ||
      build_sched(KQ_MAP_ZERO_ROW, KQ_MAP_ZERO_COL, KQ_MAP_ZERO_Q4, c->M.zero, ez, rz))
    return fail("map schedule does not fit");
  c->M.ent_gen = (const uint16_t *)dev_upload(c, eg.data(), eg.size() * 2);
  c->M.ent_zero = (const uint16_t *)dev_upload(c, ez.data(), ez.size() * 2);
  c->M.row_gen = (const uint16_t *)dev_upload(c, rg.data(), rg.size() * 2);
  c->M.row_zero = (const uint16_t *)dev_upload(c, rz.data(), rz.size() * 2);
  if (!c->M.ent_gen || !c->M.ent_zero || !c->M.row_gen || !c->M.row_zero) return fail("map upload failed");
  const char *wpb = getenv("KQED_WARPS_PER_BLOCK");
  const char *blk = getenv("KQED_BLOCKS");
  if (wpb) c->cfg.warps_per_block = std::max(1, std::min(4, atoi(wpb)));
  if (blk) c->cfg.blocks = std::max(0, atoi(blk));
  const char *nr = getenv("KQED_MIXED_NEAR");
  if (nr) c->cfg.near_ratio = std::max(1.0, std::min(64.0, atof(nr)));
  const char *orr = getenv("KQED_MIXED_ORIGIN");
  if (orr) c->cfg.origin_radius = std::max(0.0, std::min(10.0, atof(orr)));
  const char *c32 = getenv("KQED_MIXED_CHNR32");
  if (c32) c->cfg.chnr32 = atoi(c32) ? 1 : 0;
  return 0;
}

static void free_grid(struct Grid_coeffs *G)
{
  if (G->Ffm) {
    for (int a = 0; a < G->Nffa; a++) {
      if (!G->Ffm[a]) continue;
      for (int i = 0; i < G->nstpx; i++) {
        if (!G->Ffm[a][i]) continue;
        for (int j = 0; j < G->nstpy; j++) free(G->Ffm[a][i][j]);
        free(G->Ffm[a][i]);
      }
      free(G->Ffm[a]);
    }
    free(G->Ffm);
  }
  if (G->Ffp) {
    for (int a = 0; a < G->Nffa; a++) {
      if (!G->Ffp[a]) continue;
      for (int i = 0; i < G->nstpx; i++) {
        if (!G->Ffp[a][i]) continue;
        for (int j = 0; j < G->nstpy; j++) free(G->Ffp[a][i][j]);
        free(G->Ffp[a][i]);
      }
      free(G->Ffp[a]);
    }
    free(G->Ffp);
  }
  if (G->TX) { for (int i = 0; i < 23; i++) free(G->TX[i]); free(G->TX); }
  if (G->TY) { for (int i = 0; i < 14; i++) free(G->TY[i]); free(G->TY); }
  free(G->XX); free(G->YY); free(G->nfx);
}

extern "C" void free_QED_temps(struct QED_kernel_temps *t)
{
  if (!t) return;
  Ctx *c = ctx_of(t);
  if (c) {
    if (tl_stage.owner == c->id) tl_stage.reset();
    surrogate_forget(c);
    for (void *p : c->allocs) cudaFree(p);
    delete c;
    free(t->Grid.PC);
  }
  free_grid(&t->Grid);
  free(t->G8);
  memset(t, 0, sizeof(*t));
}

extern "C" int initialise(struct QED_kernel_temps *t)
{
  if (!t) return 1;
  memset(t, 0, sizeof(*t));
  const std::string lib = lib_path();
  struct Grid_coeffs *G = &t->Grid;
  int ntx = 0, nty = 0;
  if (load_ff(lib, G) ||
      load_taylor(lib, "taylorx_cksum.bin", 23, 810, &G->TX, &ntx, &G->NY_tay) ||
      load_taylor(lib, "taylory_cksum.bin", 14, 100, &G->TY, &nty, &G->NX_tay)) {
    fprintf(stderr, "%s\n", tl_err.c_str());
    free_grid(G);
    memset(t, 0, sizeof(*t));
    return 1;
  }
  /* the reference names the TAYLORX row count NtayY and TAYLORY's NtayX
     (io.c:195, :252) */
  G->NtayY = ntx;
  G->NtayX = nty;
  Ctx *c = new Ctx();
  if (setup_device(G, c)) {
    fprintf(stderr, "%s\n", tl_err.c_str());
    for (void *p : c->allocs) cudaFree(p);
    delete c;
    free_grid(G);
    memset(t, 0, sizeof(*t));
    return 1;
  }
  G->PC = (struct AVX_precomps *)calloc(1, sizeof(struct AVX_precomps));
  G->PC->Fm = c;
  /* the Dirac-trace table of the perturbative Pi-hat, as the reference's
     initialise fills it (src/LIBFILES/init.c:149-150) */
  t->G8 = (int *)malloc(65536 * sizeof(int));
  if (t->G8) init_g8(t);
  return 0;
}

extern "C" int initialize_QED_kernel_temps(struct QED_kernel_temps *t) { return initialise(t); }

/* ------------------------------------------------------ batched kernels */

static int check_variant_precision(int variant, int precision)
{
  if (variant < 0 || variant > 3) return fail("variant %d not in 0..3", variant);
  if (precision != KQED_FP64 && precision != KQED_FP32_MIXED)
    return fail("precision mode %d is not available for this entry point", precision);
  return 0;
}

/* the lattice sums also take the surrogate form, once a network is attached */
static int check_lattice_precision(Ctx *c, int variant, int precision)
{
  if (precision == KQED_SURROGATE) {
    if (variant < 0 || variant > 3) return fail("variant %d not in 0..3", variant);
    if (!surrogate_ready(c))
      return fail("precision KQED_SURROGATE: no surrogate trained for these tables "
                  "(kqed_surrogate_train)");
    return 0;
  }
  return check_variant_precision(variant, precision);
}

/* L0 over n pairs on the device */
static thread_local int tl_precision = KQED_FP64;

/* record scratch for n pairs (capped at kRecPairs; launches are chunked):
   records [cap][kRec], Pi envelopes [cap], the mixed form's deferred-record
   list [cap] + its count, codes [cap] bytes */
static int rec_scratch_in(Scratch &buf, size_t n, double **rec, uint8_t **code, size_t *cap,
                          double **env = nullptr, uint32_t **list = nullptr,
                          unsigned **count = nullptr)
{
  size_t c = std::min(std::max(n, (size_t)kTile), kRecPairs);
  c = (c + kTile - 1) / kTile * kTile;
  double *b = buf.get(c * kRec + c + c / 2 + 1 + c / 8 + 1);
  if (!b) return fail("out of device memory for %zu pair records", c);
  *rec = b;
  if (env) *env = b + c * kRec;
  if (list) *list = reinterpret_cast<uint32_t *>(b + c * kRec + c);
  if (count) *count = reinterpret_cast<unsigned *>(b + c * kRec + c + c / 2);
  *code = reinterpret_cast<uint8_t *>(b + c * kRec + c + c / 2 + 1);
  *cap = c;
  return 0;
}

static int rec_scratch(ThreadStage &st, size_t n, double **rec, uint8_t **code, size_t *cap,
                       double **env = nullptr, uint32_t **list = nullptr,
                       unsigned **count = nullptr)
{
  return rec_scratch_in(st.d_rec, n, rec, code, cap, env, list, count);
}

/* explicit record space (batch plans own theirs) */
struct RecSpace {
  double *rec;
  uint8_t *code;
  size_t cap;
};

static int run_l0(Ctx *c, const double *dx, const double *dy, size_t n, double *dout,
                  uint8_t *dstatus, cudaStream_t s, bool timed = true,
                  const RecSpace *rs = nullptr)
{
  L0Args a{dx, dy, n, dout, dstatus, nullptr, nullptr, 0};
  if (n == 0) return 0;
  if (rs) {
    a.rec = rs->rec;
    a.code = rs->code;
    a.rec_cap = rs->cap;
  } else if (rec_scratch(stage_for(c), n, &a.rec, &a.code, &a.rec_cap)) {
    return 1;
  }
  TimedLaunch tl{nullptr, nullptr};
  if (timed) prof_begin(s, tl);
  if (tl_precision == KQED_FP32_MIXED && timed) CUDA_OK(launch_l0_mixed(c->T, c->M, a, c->cfg, s));
  else CUDA_OK(launch_l0_fp64(c->T, c->M, a, c->cfg, s));
  prof_end(s, tl);
  return 0;
}

/* QED_kernel_L1/L2/L3 (src/LIBFILES/kernels.c:117-177) as L0 terms */
static int run_variant(Ctx *c, int variant, const double *dx, const double *dy, size_t n,
                       double *dout, uint8_t *dstatus, cudaStream_t s, ThreadStage &st)
{
  if (run_l0(c, dx, dy, n, dout, dstatus, s, true)) return 1;
  if (variant == 0) return 0;
  double *tmp = st.d_tmp.get(n * 384);
  double *zero = st.d_aux.get(n * 4);
  if (!tmp || !zero) return fail("out of device memory for %zu pairs", n);
  CUDA_OK(launch_fill_pairs(nullptr, n, 0, zero, s));
  switch (variant) {
  case 1:
    if (run_l0(c, dx, dx, n, tmp, nullptr, s)) return 1;
    CUDA_OK(launch_axpy(dout, tmp, -0.5, n * 384, s));
    if (run_l0(c, dy, dy, n, tmp, nullptr, s)) return 1;
    CUDA_OK(launch_axpy(dout, tmp, -0.5, n * 384, s));
    break;
  case 2:
    if (run_l0(c, zero, dy, n, tmp, nullptr, s)) return 1;
    CUDA_OK(launch_axpy(dout, tmp, -1.0, n * 384, s));
    if (run_l0(c, dx, zero, n, tmp, nullptr, s)) return 1;
    CUDA_OK(launch_axpy(dout, tmp, -1.0, n * 384, s));
    break;
  case 3:
    if (run_l0(c, dx, dx, n, tmp, nullptr, s)) return 1;
    CUDA_OK(launch_axpy(dout, tmp, -1.0, n * 384, s));
    if (run_l0(c, zero, dx, n, tmp, nullptr, s)) return 1;
    CUDA_OK(launch_axpy(dout, tmp, +1.0, n * 384, s));
    if (run_l0(c, zero, dy, n, tmp, nullptr, s)) return 1;
    CUDA_OK(launch_axpy(dout, tmp, -1.0, n * 384, s));
    break;
  }
  return 0;
}

extern "C" int kqed_kernel_batch_dev(const struct QED_kernel_temps *t, int variant, size_t n,
                                     const double *d_x, const double *d_y, double *d_kerv,
                                     uint8_t *d_status, int precision, void *stream)
{
  Ctx *c = ctx_of(t);
  if (!c) return fail("tables not initialised");
  if (check_variant_precision(variant, precision)) return 1;
  if (n && (!d_x || !d_y || !d_kerv)) return fail("null buffer");
  tl_precision = precision;
  const int rc = run_variant(c, variant, d_x, d_y, n, d_kerv, d_status, (cudaStream_t)stream, stage_for(c));
  tl_precision = KQED_FP64;
  return rc;
}

/* Error of the mixed form against the FP64 form, accumulated on the device:
   both forms of L<variant> are evaluated on chunks of pairs and compared by
   stats_kernel; only the 771 accumulators come back to the host. */
extern "C" int kqed_precision_stats(const struct QED_kernel_temps *t, int variant, size_t n,
                                    const double *d_x, const double *d_y, double floor_abs,
                                    double *stats, void *stream)
{
  Ctx *c = ctx_of(t);
  if (!c) return fail("tables not initialised");
  if (check_variant_precision(variant, KQED_FP64)) return 1;
  if (!stats) return fail("null buffer");
  for (int i = 0; i < KQED_STATS_LEN; i++) stats[i] = 0.0;
  if (n == 0) return 0;
  if (!d_x || !d_y) return fail("null buffer");
  if (!(floor_abs > 0.0)) return fail("floor must be positive");
  cudaStream_t s = (cudaStream_t)stream;
  ThreadStage &st = stage_for(c);
  const size_t chunk = std::min(n, (size_t)1 << 18);
  double *A = st.d_sa.get(chunk * 384 + 771);
  double *B = st.d_sb.get(chunk * 384);
  if (!A || !B) return fail("out of device memory for %zu-pair statistics chunks", chunk);
  double *acc = A + chunk * 384;
  CUDA_OK(cudaMemsetAsync(acc, 0, 771 * sizeof(double), s));
  for (size_t p0 = 0; p0 < n; p0 += chunk) {
    const size_t m = std::min(chunk, n - p0);
    tl_precision = KQED_FP64;
    int bad = run_variant(c, variant, d_x + 4 * p0, d_y + 4 * p0, m, A, nullptr, s, st);
    tl_precision = KQED_FP32_MIXED;
    bad = bad || run_variant(c, variant, d_x + 4 * p0, d_y + 4 * p0, m, B, nullptr, s, st);
    tl_precision = KQED_FP64;
    if (bad) return 1;
    CUDA_OK(launch_stats(A, B, m, floor_abs, acc, s));
  }
  double h[771];
  CUDA_OK(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
  CUDA_OK(cudaStreamSynchronize(s));
  const double cnt = h[770];
  for (int i = 0; i < 384; i++) {
    stats[i] = h[i];
    stats[384 + i] = cnt > 0 ? std::sqrt(h[384 + i] / cnt) : 0.0;
  }
  stats[768] = h[768];
  stats[769] = cnt > 0 ? h[769] / cnt : 0.0;
  stats[770] = cnt;
  return 0;
}

extern "C" int kqed_kernel_batch(const struct QED_kernel_temps *t, int variant, size_t n,
                                 const double *x, const double *y, double *kerv, uint8_t *status,
                                 int precision)
{
  Ctx *c = ctx_of(t);
  if (!c) return fail("tables not initialised");
  if (check_variant_precision(variant, precision)) return 1;
  if (n == 0) return 0;
  if (!x || !y || !kerv) return fail("null buffer");
  if (n > SIZE_MAX / (sizeof(double) * (8 + 384 + 1))) return fail("%zu pairs do not fit the address space", n);
  ThreadStage &st = stage_for(c);
  if (!st.stream) CUDA_OK(cudaStreamCreateWithFlags(&st.stream, cudaStreamNonBlocking));
  /* an output in kqed_pinned_alloc memory is written in place by the kernels
     (no device copy, no copy back) */
  double *kin = static_cast<double *>(kqed::pinned_device(kerv, n * 384 * sizeof(double)));
  const size_t nk = kin ? 0 : n * 384;
  double *io = st.d_io.get(n * 8 + nk + (n + 7) / 8);
  if (!io) return fail("out of device memory for %zu pairs", n);
  double *dx = io, *dy = io + 4 * n, *dk = kin ? kin : io + 8 * n;
  uint8_t *dst = status ? reinterpret_cast<uint8_t *>(io + n * 8 + nk) : nullptr;
  CUDA_OK(cudaMemcpyAsync(dx, x, n * 4 * sizeof(double), cudaMemcpyHostToDevice, st.stream));
  CUDA_OK(cudaMemcpyAsync(dy, y, n * 4 * sizeof(double), cudaMemcpyHostToDevice, st.stream));
  tl_precision = precision;
  const int rc = run_variant(c, variant, dx, dy, n, dk, dst, st.stream, st);
  tl_precision = KQED_FP64;
  if (rc) return 1;
  if (!kin)
    CUDA_OK(cudaMemcpyAsync(kerv, dk, n * 384 * sizeof(double), cudaMemcpyDeviceToHost, st.stream));
  if (status) CUDA_OK(cudaMemcpyAsync(status, dst, n, cudaMemcpyDeviceToHost, st.stream));
  CUDA_OK(cudaStreamSynchronize(st.stream));
  return 0;
}

/* ---------------------------------------------------- legacy per pair */

static void legacy(int variant, const double xv[4], const double yv[4],
                   const struct QED_kernel_temps &t, double kerv[6][4][4][4])
{
  double *out = &kerv[0][0][0][0];
  Ctx *c = ctx_of(&t);
  if (!c) {
    fprintf(stderr, "QED_kernel_L%d: tables not initialised\n", variant);
    memset(out, 0, 384 * sizeof(double));
    return;
  }
  ThreadStage &st = stage_for(c);
  if (!st.h_pin) {
    if (cudaMallocHost(&st.h_pin, (8 + 384) * sizeof(double)) != cudaSuccess) st.h_pin = nullptr;
  }
  if (!st.stream) cudaStreamCreateWithFlags(&st.stream, cudaStreamNonBlocking);
  double *io = st.d_io.get(8 + 384 + 1);
  if (!st.h_pin || !st.stream || !io) {
    fprintf(stderr, "QED_kernel_L%d: GPU staging unavailable\n", variant);
    memset(out, 0, 384 * sizeof(double));
    return;
  }
  memcpy(st.h_pin, xv, 4 * sizeof(double));
  memcpy(st.h_pin + 4, yv, 4 * sizeof(double));
  int err = cudaMemcpyAsync(io, st.h_pin, 8 * sizeof(double), cudaMemcpyHostToDevice, st.stream) != cudaSuccess;
  if (!err) err = run_variant(c, variant, io, io + 4, 1, io + 8, nullptr, st.stream, st);
  if (!err)
    err = cudaMemcpyAsync(st.h_pin + 8, io + 8, 384 * sizeof(double), cudaMemcpyDeviceToHost, st.stream) != cudaSuccess;
  if (!err) err = cudaStreamSynchronize(st.stream) != cudaSuccess;
  if (err) {
    fprintf(stderr, "QED_kernel_L%d: %s\n", variant, tl_err.c_str());
    memset(out, 0, 384 * sizeof(double));
    return;
  }
  memcpy(out, st.h_pin + 8, 384 * sizeof(double));
}

extern "C" void QED_kernel_L0(const double xv[4], const double yv[4], const struct QED_kernel_temps t,
                              double kerv[6][4][4][4])
{
  legacy(0, xv, yv, t, kerv);
}
extern "C" void QED_kernel_L1(const double xv[4], const double yv[4], const struct QED_kernel_temps t,
                              double kerv[6][4][4][4])
{
  legacy(1, xv, yv, t, kerv);
}
extern "C" void QED_kernel_L2(const double xv[4], const double yv[4], const struct QED_kernel_temps t,
                              double kerv[6][4][4][4])
{
  legacy(2, xv, yv, t, kerv);
}
extern "C" void QED_kernel_L3(const double xv[4], const double yv[4], const struct QED_kernel_temps t,
                              double kerv[6][4][4][4])
{
  legacy(3, xv, yv, t, kerv);
}

/* ------------------------------------------------------- lattice sums */

/* per-site and per-x additive kernel terms of L1..L3 for the fused sum:
   Lv(x,y) = L0(x,y) + Ky(y) + Bx(x) */
static int lattice_terms(Ctx *c, int variant, const double *dx, size_t nx, const double *dy,
                         size_t ny, double **Ky, double **Bx, cudaStream_t s, ThreadStage &st)
{
  *Ky = *Bx = nullptr;
  if (variant == 0) return 0;
  double *ky = st.d_aux.get(ny * 384 + ny * 4);
  double *bx = st.d_aux2.get(nx * 384 * 2 + nx * 4);
  if (!ky || !bx) return fail("out of device memory for lattice terms");
  double *zy = ky + ny * 384;          /* ny zero vectors */
  double *bt = bx + nx * 384;          /* nx*384 temporary */
  double *zx = bt + nx * 384;          /* nx zero vectors */
  CUDA_OK(launch_fill_pairs(nullptr, ny, 0, zy, s));
  CUDA_OK(launch_fill_pairs(nullptr, nx, 0, zx, s));
  switch (variant) {
  case 1: /* L1 = L0(x,y) - L0(x,x)/2 - L0(y,y)/2 */
    if (run_l0(c, dy, dy, ny, ky, nullptr, s, false) || run_l0(c, dx, dx, nx, bx, nullptr, s, false)) return 1;
    CUDA_OK(launch_scale(ky, -0.5, ny * 384, s));
    CUDA_OK(launch_scale(bx, -0.5, nx * 384, s));
    break;
  case 2: /* L2 = L0(x,y) - L0(0,y) - L0(x,0) */
    if (run_l0(c, zy, dy, ny, ky, nullptr, s, false) || run_l0(c, dx, zx, nx, bx, nullptr, s, false)) return 1;
    CUDA_OK(launch_scale(ky, -1.0, ny * 384, s));
    CUDA_OK(launch_scale(bx, -1.0, nx * 384, s));
    break;
  case 3: /* L3 = L0(x,y) - L0(x,x) + L0(0,x) - L0(0,y) */
    if (run_l0(c, zy, dy, ny, ky, nullptr, s, false) || run_l0(c, dx, dx, nx, bx, nullptr, s, false) ||
        run_l0(c, zx, dx, nx, bt, nullptr, s, false))
      return 1;
    CUDA_OK(launch_scale(ky, -1.0, ny * 384, s));
    CUDA_OK(launch_scale(bx, -1.0, nx * 384, s));
    CUDA_OK(launch_axpy(bx, bt, 1.0, nx * 384, s));
    break;
  }
  *Ky = ky;
  *Bx = bx;
  return 0;
}

/* state of one fused lattice sum between its preparation, its per-x-chunk
   launches and the final reduction */
struct LatticeRun {
  Ctx *c;
  const double *d_x, *d_y;
  size_t nx, ny;
  double *Ky, *Bx, *partial, *col, *rec, *env;
  uint32_t *list;
  unsigned *count;
  float2 *Ky2, *Bx2;
  float *col32;
  float2 *coldf;
  uint8_t *code;
  size_t rec_cap;
  int tiles, precision, variant;
  uint64_t pi_seed;       /* generated Pi (lattice_launch with d_pi == NULL) */
  uint32_t pi_stream;
  size_t x_offset, y_offset;   /* generated Pi: global indices of x[0], y[0] */
  int asm_blocks;              /* > 0: the assembly kernels' grid (else the tuned one) */
};

static int lattice_prepare(Ctx *c, int variant, size_t nx, const double *d_x, size_t ny,
                           const double *d_y, cudaStream_t s, ThreadStage &st, LatticeRun &R,
                           int precision)
{
  R.c = c; R.d_x = d_x; R.d_y = d_y; R.nx = nx; R.ny = ny; R.precision = precision;
  R.variant = variant;
  R.pi_seed = 0;
  R.pi_stream = 0;
  R.x_offset = R.y_offset = 0;
  R.asm_blocks = 0;
  R.Ky2 = R.Bx2 = nullptr;
  R.col32 = nullptr;
  R.coldf = nullptr;
  R.col = nullptr;
  R.tiles = (int)((ny + kTile - 1) / kTile);
  /* records first: the kernel-term launches below reuse the same scratch */
  if (rec_scratch(st, nx * (size_t)R.tiles * kTile, &R.rec, &R.code, &R.rec_cap, &R.env,
                  &R.list, &R.count))
    return 1;
  if (lattice_terms(c, variant, d_x, nx, d_y, ny, &R.Ky, &R.Bx, s, st)) return 1;
  R.partial = st.d_tmp.get(nx * (size_t)std::max(R.tiles, 1) * 2);
  if (!R.partial) return fail("out of device memory for partial sums");
  const size_t ncol = nx * (size_t)c->T.nstpy * c->T.NK * kRow;
  const bool mixed = precision == KQED_FP32_MIXED || precision == KQED_SURROGATE;
  /* FP64 columns always (the FP64 form, and the float form's pairs near
     cb = +-1 or assembled in FP64); float columns for the float
     interpolation of the mixed form */
  R.col = st.d_col.get(ncol);
  if (!R.col) return fail("out of device memory for x-column tables");
  CUDA_OK(launch_build_columns(c->T, d_x, nx, R.col, s));
  {
    /* float tables: the mixed form's float columns (ncol floats) or the FP64
       form's (hi, lo) copy of its columns (ncol float2), an even count of
       floats (kRow = 28 per row) so the float2 tables after them stay
       8-byte aligned; then the per-site / per-x terms as float2 (both forms:
       the FP64 form contracts in double-float) */
    const size_t ncf = mixed ? ncol : 2 * ncol;
    const size_t n32 = ncf + (R.Ky ? (ny + nx) * 384 * 2 : 0);
    float *b32 = reinterpret_cast<float *>(st.d_col32.get(n32 / 2 + 2));
    if (!b32) return fail("out of device memory for float tables");
    if (mixed) {
      R.col32 = b32;
      CUDA_OK(launch_build_columns32(c->T, d_x, nx, R.col32, s));
    } else {
      R.coldf = reinterpret_cast<float2 *>(b32);
      CUDA_OK(launch_to_float2(R.col, R.coldf, ncol, s));
    }
    b32 += ncf;
    if (R.Ky) {
      /* the FP64-evaluated per-site / per-x terms, as float (hi, lo) pairs */
      R.Ky2 = reinterpret_cast<float2 *>(b32);
      R.Bx2 = R.Ky2 + ny * 384;
      CUDA_OK(launch_to_float2(R.Ky, R.Ky2, ny * 384, s));
      CUDA_OK(launch_to_float2(R.Bx, R.Bx2, nx * 384, s));
    }
  }
  return 0;
}

/* fused kernel for x points [x0, x0+nxc) with their Pi block at d_pi */
static int lattice_launch(const LatticeRun &R, size_t x0, size_t nxc, const double *d_pi,
                          cudaStream_t s)
{
  const size_t per_x = (size_t)R.c->T.nstpy * R.c->T.NK * kRow;
  const bool mixed = R.precision == KQED_FP32_MIXED;
  const bool sur = R.precision == KQED_SURROGATE;
  LatticeArgs a{};
  a.x = R.d_x + 4 * x0;
  a.y = R.d_y;
  a.nx = nxc;
  a.ny = R.ny;
  a.pi = d_pi;
  a.Ky = R.Ky;
  a.Bx = R.Bx ? R.Bx + 384 * x0 : nullptr;
  a.partial = R.partial + 2 * x0 * (size_t)std::max(R.tiles, 1);
  a.tiles = R.tiles;
  a.col = R.col ? R.col + per_x * x0 : nullptr;
  a.Ky2 = R.Ky2;
  a.Bx2 = R.Bx2 ? R.Bx2 + 384 * x0 : nullptr;
  a.col32 = R.col32 ? R.col32 + per_x * x0 : nullptr;
  a.coldf = R.coldf ? R.coldf + per_x * x0 : nullptr;
  a.rec = R.rec;
  a.code = R.code;
  a.rec_cap = R.rec_cap;
  a.env = R.env;
  a.list = R.list;
  a.count = R.count;
  a.pi_seed = R.pi_seed;
  a.pi_stream = R.pi_stream;
  a.k0 = R.x_offset + x0;
  a.n0 = R.y_offset;
  a.zero_x_vanishes = R.variant >= 2;
  LaunchCfg cfg = R.c->cfg;
  if (R.asm_blocks > 0) cfg.blocks = R.asm_blocks;
  TimedLaunch tl;
  prof_begin(s, tl);
  if (sur) {
    SurHook hook;
    if (surrogate_hook(R.c, R.rec_cap, &hook)) return 1;
    CUDA_OK(launch_lattice_surrogate(R.c->T, R.c->M, a, cfg, hook, s));
  } else if (mixed) {
    CUDA_OK(launch_lattice_mixed(R.c->T, R.c->M, a, cfg, s));
  } else {
    CUDA_OK(launch_lattice_fp64(R.c->T, R.c->M, a, cfg, s));
  }
  prof_end(s, tl);
  return 0;
}

/* Two record buffers and two streams over chunks of x (one record pass
   each): the records of one chunk are built while the assembly of the
   previous chunk runs; blocks_per_sm > 0 caps the assembly grid so that
   record blocks fit beside it.  pi: the Pi of x[0] (chunk x0 reads
   pi + x0 * per_x).  Work enqueued on s after the call follows all of it.
   (The surrogate form's network scratch is per context: one stream.) */
static int lattice_pipeline(ThreadStage &st, LatticeRun &R, size_t nx, const double *pi,
                            size_t per_x, int precision, cudaStream_t s, int blocks_per_sm)
{
  if (!pi) return fail("the chunked lattice sum needs a stored Pi");   /* (generated Pi: lattice_launch) */
  if (!st.copy_stream) CUDA_OK(cudaStreamCreateWithFlags(&st.copy_stream, cudaStreamNonBlocking));
  const bool two = precision != KQED_SURROGATE;
  LatticeRun R2 = R;
  if (two && rec_scratch_in(st.d_rec2, nx * (size_t)R.tiles * kTile, &R2.rec, &R2.code,
                            &R2.rec_cap, &R2.env, &R2.list, &R2.count))
    return 1;
  const size_t per_x_pairs = (size_t)R.tiles * kTile;
  const size_t xc = two ? std::max((size_t)1, std::min(R.rec_cap, R2.rec_cap) / per_x_pairs) : nx;
  if (xc < nx && blocks_per_sm > 0) {
    int dev = 0, sms = 0;
    CUDA_OK(cudaGetDevice(&dev));
    CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    R.asm_blocks = R2.asm_blocks = blocks_per_sm * std::max(sms, 1);
  }
  if (!st.ev_copied[0]) {
    for (int i = 0; i < 2; i++) {
      CUDA_OK(cudaEventCreateWithFlags(&st.ev_copied[i], cudaEventDisableTiming));
      CUDA_OK(cudaEventCreateWithFlags(&st.ev_free[i], cudaEventDisableTiming));
    }
  }
  cudaStream_t s2 = st.copy_stream;
  CUDA_OK(cudaEventRecord(st.ev_copied[0], s));
  CUDA_OK(cudaStreamWaitEvent(s2, st.ev_copied[0], 0));
  size_t i = 0;
  for (size_t x0 = 0; x0 < nx; x0 += xc, i++)
    if (lattice_launch((i & 1) ? R2 : R, x0, std::min(xc, nx - x0), pi + x0 * per_x,
                       (i & 1) ? s2 : s))
      return 1;
  CUDA_OK(cudaEventRecord(st.ev_free[0], s2));
  CUDA_OK(cudaStreamWaitEvent(s, st.ev_free[0], 0));
  return 0;
}

extern "C" int kqed_lattice_sum_dev(const struct QED_kernel_temps *t, int variant, size_t nx,
                                    const double *d_x, size_t ny, const double *d_y,
                                    const double *d_pi, double *d_sums, int precision, void *stream)
{
  Ctx *c = ctx_of(t);
  if (!c) return fail("tables not initialised");
  if (check_lattice_precision(c, variant, precision)) return 1;
  if (nx == 0) return 0;
  if (!d_sums) return fail("null buffer");
  cudaStream_t s = (cudaStream_t)stream;
  if (ny == 0) {   /* an empty lattice sums to zero (its site and Pi pointers may be NULL) */
    CUDA_OK(cudaMemsetAsync(d_sums, 0, nx * sizeof(double), s));
    return 0;
  }
  if (!d_x || !d_y || !d_pi) return fail("null buffer");
  ThreadStage &st = stage_for(c);
  LatticeRun R;
  if (lattice_prepare(c, variant, nx, d_x, ny, d_y, s, st, R, precision)) return 1;
  /* the mixed form overlaps one chunk's records with the previous chunk's
     assembly (24^4 lattice, 32 x: 44.2 -> 42.4 ms per call); in the FP64
     form the overlap was slower (137.3 ms in sequence, 140.9 overlapped) */
  if (precision == KQED_FP32_MIXED) {
    if (lattice_pipeline(st, R, nx, d_pi, ny * 384, precision, s, 0)) return 1;
  } else if (lattice_launch(R, 0, nx, d_pi, s)) {
    return 1;
  }
  CUDA_OK(launch_reduce_partials(R.partial, nx, R.tiles, d_sums, s));
  return 0;
}

extern "C" int kqed_lattice_sum_synth(const struct QED_kernel_temps *t, int variant, size_t nx,
                                      const double *d_x, size_t ny, const double *d_y,
                                      uint64_t seed, uint32_t stream_id, size_t x_offset,
                                      size_t y_offset, double *d_sums, int precision,
                                      void *stream)
{
  Ctx *c = ctx_of(t);
  if (!c) return fail("tables not initialised");
  if (check_lattice_precision(c, variant, precision)) return 1;
  if (nx == 0) return 0;
  if (!d_sums) return fail("null buffer");
  cudaStream_t s = (cudaStream_t)stream;
  if (ny == 0) {   /* an empty lattice sums to zero (its site pointer may be NULL) */
    CUDA_OK(cudaMemsetAsync(d_sums, 0, nx * sizeof(double), s));
    return 0;
  }
  if (!d_x || !d_y) return fail("null buffer");
  ThreadStage &st = stage_for(c);
  LatticeRun R;
  if (lattice_prepare(c, variant, nx, d_x, ny, d_y, s, st, R, precision)) return 1;
  R.pi_seed = seed;
  R.pi_stream = stream_id;
  R.x_offset = x_offset;
  R.y_offset = y_offset;
  if (lattice_launch(R, 0, nx, nullptr, s)) return 1;
  CUDA_OK(launch_reduce_partials(R.partial, nx, R.tiles, d_sums, s));
  return 0;
}

extern "C" int kqed_pi_synth_dev(size_t nx, const double *d_x, size_t ny, const double *d_y,
                                 uint64_t seed, uint32_t stream_id, size_t x_offset,
                                 size_t y_offset, double *d_pi, void *stream)
{
  if (nx == 0 || ny == 0) return 0;
  if (!d_x || !d_y || !d_pi) return fail("null buffer");
  CUDA_OK(launch_pi_synth(d_x, nx, d_y, ny, seed, stream_id, x_offset, y_offset, d_pi,
                          (cudaStream_t)stream));
  return 0;
}

/* the device address of [p, p + bytes) when the whole range lies in one
   allocation of kqed_pinned_alloc (page-locked and mapped), else null */
static const void *pinned_device_range(const void *p, size_t bytes);

/* KQED_HOST_PI=copy: stage Pi through device buffers even when the kernels
   could read it in place */
static bool host_pi_copy_forced()
{
  const char *v = getenv("KQED_HOST_PI");
  return v && strcmp(v, "copy") == 0;
}

/* Host buffers.  Pi in memory from kqed_pinned_alloc is read in place by the
   kernels over the host link (Grace's NVLink-C2C carries the GPU's loads of
   page-locked host memory; no staging copies, and no copy-engine warm-up:
   on the GB300 machines a 32.6 GB Pi ran at 200 ms per FP64 step in place
   against 240-280 ms staged).  Other host memory streams to the device in
   per-x chunks through a double buffer on a copy stream, so the transfer of
   chunk i+1 overlaps the fused kernel on chunk i (with pinned host memory
   the copies run asynchronously).  The sums are the same either way, bit
   for bit. */
extern "C" int kqed_lattice_sum(const struct QED_kernel_temps *t, int variant, size_t nx,
                                const double *x, size_t ny, const double *y, const double *pi,
                                double *sums, int precision)
{
  Ctx *c = ctx_of(t);
  if (!c) return fail("tables not initialised");
  if (check_lattice_precision(c, variant, precision)) return 1;
  if (nx == 0) return 0;
  if (!sums) return fail("null buffer");
  if (ny == 0) {   /* an empty lattice sums to zero (its site and Pi pointers may be NULL) */
    for (size_t k = 0; k < nx; k++) sums[k] = 0.0;
    return 0;
  }
  if (!x || !y || !pi) return fail("null buffer");
  ThreadStage &st = stage_for(c);
  if (!st.stream) CUDA_OK(cudaStreamCreateWithFlags(&st.stream, cudaStreamNonBlocking));
  if (!st.copy_stream) CUDA_OK(cudaStreamCreateWithFlags(&st.copy_stream, cudaStreamNonBlocking));
  const size_t per_x = ny * 384;
  if (per_x / 384 != ny || (nx * per_x) / per_x != nx || nx * per_x > SIZE_MAX / sizeof(double))
    return fail("Pi of %zu x %zu x 384 doubles does not fit the address space", nx, ny);
  const void *pi_dev = host_pi_copy_forced()
                           ? nullptr
                           : pinned_device_range(pi, nx * per_x * sizeof(double));
  if (pi_dev) {
    double *io = st.d_io.get(nx * 5 + ny * 4);
    if (!io) return fail("out of device memory for %zu x %zu pairs", nx, ny);
    double *dx = io, *dy = io + nx * 4, *ds = dy + ny * 4;
    cudaStream_t s = st.stream;
    CUDA_OK(cudaMemcpyAsync(dx, x, nx * 4 * sizeof(double), cudaMemcpyHostToDevice, s));
    CUDA_OK(cudaMemcpyAsync(dy, y, ny * 4 * sizeof(double), cudaMemcpyHostToDevice, s));
    LatticeRun R;
    if (lattice_prepare(c, variant, nx, dx, ny, dy, s, st, R, precision)) return 1;
    /* Only the assembly reads Pi: the records of one chunk of x are built
       on a second stream while the assembly of the previous chunk reads its
       Pi, so the host link stays busy; the assembly grid is capped at 4
       blocks per SM, which leaves room on every SM for record blocks (24^4
       lattice, 32 x: FP64 213 ms per call with one stream, 200 ms so; mixed
       173 and 160 ms). */
    if (lattice_pipeline(st, R, nx, static_cast<const double *>(pi_dev), per_x, precision, s, 4))
      return 1;
    CUDA_OK(launch_reduce_partials(R.partial, nx, R.tiles, ds, s));
    CUDA_OK(cudaMemcpyAsync(sums, ds, nx * sizeof(double), cudaMemcpyDeviceToHost, s));
    CUDA_OK(cudaStreamSynchronize(s));
    return 0;
  }
  /* chunk of about 128 M doubles (1 GB) of Pi, at least one x */
  size_t nxc = std::max((size_t)1, ((size_t)128 << 20) / std::max(per_x, (size_t)1));
  nxc = std::min(nxc, nx);
  double *io = st.d_io.get(nx * 5 + ny * 4 + 2 * nxc * per_x);
  if (!io) return fail("out of device memory for %zu x %zu pairs", nx, ny);
  double *dx = io, *dy = io + nx * 4, *ds = dy + ny * 4, *slot[2] = {ds + nx, ds + nx + nxc * per_x};
  cudaStream_t s = st.stream, cs = st.copy_stream;
  CUDA_OK(cudaMemcpyAsync(dx, x, nx * 4 * sizeof(double), cudaMemcpyHostToDevice, s));
  CUDA_OK(cudaMemcpyAsync(dy, y, ny * 4 * sizeof(double), cudaMemcpyHostToDevice, s));
  LatticeRun R;
  if (lattice_prepare(c, variant, nx, dx, ny, dy, s, st, R, precision)) return 1;
  if (!st.ev_copied[0]) {
    for (int i = 0; i < 2; i++) {
      CUDA_OK(cudaEventCreateWithFlags(&st.ev_copied[i], cudaEventDisableTiming));
      CUDA_OK(cudaEventCreateWithFlags(&st.ev_free[i], cudaEventDisableTiming));
    }
  }
  const size_t nchunks = (nx + nxc - 1) / nxc;
  for (size_t ch = 0; ch < nchunks; ch++) {
    const int b = (int)(ch & 1);
    const size_t x0 = ch * nxc, n = std::min(nxc, nx - x0);
    if (ch >= 2) CUDA_OK(cudaStreamWaitEvent(cs, st.ev_free[b], 0));
    TimedLaunch tc;
    prof_begin(cs, tc, 1);
    CUDA_OK(cudaMemcpyAsync(slot[b], pi + x0 * per_x, n * per_x * sizeof(double),
                            cudaMemcpyHostToDevice, cs));
    prof_end(cs, tc);
    CUDA_OK(cudaEventRecord(st.ev_copied[b], cs));
    CUDA_OK(cudaStreamWaitEvent(s, st.ev_copied[b], 0));
    if (lattice_launch(R, x0, n, slot[b], s)) return 1;
    CUDA_OK(cudaEventRecord(st.ev_free[b], s));
  }
  CUDA_OK(launch_reduce_partials(R.partial, nx, R.tiles, ds, s));
  CUDA_OK(cudaMemcpyAsync(sums, ds, nx * sizeof(double), cudaMemcpyDeviceToHost, s));
  CUDA_OK(cudaStreamSynchronize(s));
  return 0;
}

/* --------------------------------------------- pinned host buffers */

/* Page-locked host memory for a caller's Pi (or any input of the host entry
   points), allocated with cudaHostAlloc: host-to-device copies from it run
   at the full host link rate (about 211 GB/s on the GB300 machines, Grace's
   NVLink-C2C), which memory pinned by other allocators did not always
   reach. */
/* The library's page-locked allocations: host address -> (bytes, device
   address), so that the host entry points can tell whether a caller's
   buffer lies wholly inside one of them. */
static std::mutex g_pinned_mu;
static std::map<uintptr_t, std::pair<size_t, uintptr_t>> g_pinned;

extern "C" int kqed_pinned_alloc(size_t bytes, void **ptr)
{
  if (!ptr) return fail("null buffer");
  *ptr = nullptr;
  if (bytes == 0) return 0;
  if (cudaHostAlloc(ptr, bytes, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
    *ptr = nullptr;
    return fail("cudaHostAlloc of %zu bytes failed", bytes);
  }
  void *dev = nullptr;
  if (cudaHostGetDevicePointer(&dev, *ptr, 0) != cudaSuccess) dev = nullptr;
  std::lock_guard<std::mutex> lk(g_pinned_mu);
  g_pinned[(uintptr_t)*ptr] = {bytes, (uintptr_t)dev};
  return 0;
}

extern "C" int kqed_pinned_free(void *ptr)
{
  if (!ptr) return 0;
  {
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    g_pinned.erase((uintptr_t)ptr);
  }
  if (cudaFreeHost(ptr) != cudaSuccess) return fail("cudaFreeHost failed");
  return 0;
}

static const void *pinned_device_range(const void *p, size_t bytes)
{
  if (!p || bytes == 0) return nullptr;
  const uintptr_t a = (uintptr_t)p;
  std::lock_guard<std::mutex> lk(g_pinned_mu);
  auto it = g_pinned.upper_bound(a);
  if (it == g_pinned.begin()) return nullptr;
  --it;
  const uintptr_t base = it->first;
  const size_t size = it->second.first;
  const uintptr_t dev = it->second.second;
  if (!dev || a - base > size || bytes > size - (a - base)) return nullptr;
  /* the driver must still see both ends as page-locked memory mapped where
     the registry says (a block released by cudaFreeHost instead of
     kqed_pinned_free leaves a stale entry; such memory is staged instead) */
  const uintptr_t ends[2] = {a, a + bytes - 1};
  for (uintptr_t e : ends) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, (const void *)e) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    if (pa.type != cudaMemoryTypeHost || (uintptr_t)pa.devicePointer != dev + (e - base))
      return nullptr;
  }
  return (const void *)(dev + (a - base));
}

extern "C" int kqed_pinned_contains(const void *ptr, size_t bytes)
{
  return pinned_device_range(ptr, bytes) ? 1 : 0;
}

/* ---------------------------------------------- multi-GPU sharding */

/* Rank `rank` of `world` takes sites [*begin, *end): contiguous slabs of
   whole 64-site tiles, sizes differing by at most one tile (the slabs of
   kqed_gb300/shard.py).  Every rank evaluates its slab against all x
   (kqed_lattice_sum_dev on the slab, or kqed_lattice_sum_synth with
   y_offset = *begin); the per-x partial sums are then gathered and added by
   kqed_shard_combine. */
extern "C" int kqed_shard_slab(size_t ny, int rank, int world, size_t *begin, size_t *end)
{
  if (!begin || !end) return fail("null buffer");
  if (world < 1 || rank < 0 || rank >= world) return fail("rank %d not in a world of %d", rank, world);
  const size_t tiles = (ny + kTile - 1) / kTile;
  const size_t lo = (size_t)rank * tiles / (size_t)world, hi = (size_t)(rank + 1) * tiles / (size_t)world;
  *begin = std::min(lo * kTile, ny);
  *end = std::min(hi * kTile, ny);
  return 0;
}

/* sums[k] = compensated (Neumaier) sum over ranks r = 0 .. world-1, in rank
   order, of parts[r][k]: the result does not depend on the order in which a
   collective delivered the parts */
extern "C" int kqed_shard_combine(size_t nx, int world, const double *parts, double *sums)
{
  if (world < 1) return fail("world %d", world);
  if (nx && (!parts || !sums)) return fail("null buffer");
  for (size_t k = 0; k < nx; k++) {
    double sm = 0.0, c = 0.0;
    for (int r = 0; r < world; r++) {
      const double p = parts[(size_t)r * nx + k], t = sm + p;
      c += std::fabs(sm) >= std::fabs(p) ? (sm - t) + p : (p - t) + sm;
      sm = t;
    }
    sums[k] = sm + c;
  }
  return 0;
}

/* ---------------------------------------------- internal accessors */

namespace kqed {

int ctx_handles(const struct QED_kernel_temps *t, DevTables *T, DevMaps *M, LaunchCfg *cfg)
{
  Ctx *c = ctx_of(t);
  if (!c) return 1;
  *T = c->T;
  *M = c->M;
  *cfg = c->cfg;
  return 0;
}

int set_error(const char *msg)
{
  tl_err = msg;
  return 1;
}

int l0_pairs(const struct QED_kernel_temps *t, const double *dx, const double *dy, size_t n,
             double *dout, int precision, cudaStream_t s)
{
  Ctx *c = ctx_of(t);
  if (!c) return fail("tables not initialised");
  if (check_variant_precision(0, precision)) return 1;
  tl_precision = precision;
  const int rc = run_l0(c, dx, dy, n, dout, nullptr, s, true);
  tl_precision = KQED_FP64;
  return rc;
}

double *stage_scratch(const struct QED_kernel_temps *t, int slot, size_t n)
{
  Ctx *c = ctx_of(t);
  if (!c) return nullptr;
  ThreadStage &st = stage_for(c);
  return slot == 0 ? st.d_cmp.get(n) : st.d_cmp_io.get(n);
}

cudaStream_t stage_stream(const struct QED_kernel_temps *t)
{
  Ctx *c = ctx_of(t);
  if (!c) return nullptr;
  ThreadStage &st = stage_for(c);
  if (!st.stream) cudaStreamCreateWithFlags(&st.stream, cudaStreamNonBlocking);
  return st.stream;
}

void *pinned_device(const void *p, size_t bytes)
{
  return const_cast<void *>(pinned_device_range(p, bytes));
}

} // namespace kqed

/* ------------------------------------------------- batched lattices */

/* A batch of fused lattice sums as one work list: every lattice (job)
   contributes its units (one x, kTile sites) to a single unit list, so one
   record kernel and one assembly kernel per record chunk serve all jobs.
   The plan owns every buffer the batch needs, runs the batch once eagerly
   (choosing launch parameters when asked to tune), and captures the whole
   sequence -- column tables, per-site / per-x kernel terms, the two
   kernels, the per-job reductions -- in one CUDA graph that
   kqed_batch_plan_launch replays. */
struct kqed_batch_plan {
  Ctx *c = nullptr;
  int precision = KQED_FP64;
  std::vector<kqed_lattice_job> jobs;
  std::vector<LatticeArgs> hj;      /* device-side descriptors, host copy */
  LatticeArgs *d_jobs = nullptr;
  LatticeArgs shared{};             /* carries the record scratch */
  RecSpace rs{};
  size_t units = 0;
  LaunchCfg cfg{};
  std::vector<void *> allocs;
  /* per-site terms shared by jobs with the same site array and term kind */
  struct YTerm { const double *d_y; size_t ny; int kind; double *ky; float2 *ky2; };
  std::vector<YTerm> yterms;
  std::vector<double *> bx, bt;     /* per job */
  std::vector<float2 *> bx2;
  double *zeros = nullptr;          /* max(nx, ny) zero 4-vectors */
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t graph_kernels = 0;
  double tuned_ms = 0.0;
};

namespace {

template <typename P> int plan_alloc(kqed_batch_plan *p, P **out, size_t count)
{
  void *m = nullptr;
  if (cudaMalloc(&m, std::max(count, (size_t)1) * sizeof(P)) != cudaSuccess)
    return fail("out of device memory for a lattice batch plan (%zu bytes)", count * sizeof(P));
  p->allocs.push_back(m);
  *out = static_cast<P *>(m);
  return 0;
}

/* term kind of the per-site part: 1 = -L0(y,y)/2 (L1), 2 = -L0(0,y) (L2, L3) */
int yterm_kind(int variant) { return variant == 1 ? 1 : 2; }

int plan_enqueue_terms(kqed_batch_plan *p, cudaStream_t s)
{
  Ctx *c = p->c;
  const bool mixed = p->precision == KQED_FP32_MIXED;
  for (auto &Y : p->yterms) {
    if (Y.kind == 1) {
      if (run_l0(c, Y.d_y, Y.d_y, Y.ny, Y.ky, nullptr, s, false, &p->rs)) return 1;
      CUDA_OK(launch_scale(Y.ky, -0.5, Y.ny * 384, s));
    } else {
      if (run_l0(c, p->zeros, Y.d_y, Y.ny, Y.ky, nullptr, s, false, &p->rs)) return 1;
      CUDA_OK(launch_scale(Y.ky, -1.0, Y.ny * 384, s));
    }
    CUDA_OK(launch_to_float2(Y.ky, Y.ky2, Y.ny * 384, s));
  }
  for (size_t j = 0; j < p->jobs.size(); j++) {
    const kqed_lattice_job &J = p->jobs[j];
    double *bx = p->bx[j];
    switch (J.variant) {
    case 0:
      continue;
    case 1: /* -L0(x,x)/2 */
      if (run_l0(c, J.d_x, J.d_x, J.nx, bx, nullptr, s, false, &p->rs)) return 1;
      CUDA_OK(launch_scale(bx, -0.5, J.nx * 384, s));
      break;
    case 2: /* -L0(x,0) */
      if (run_l0(c, J.d_x, p->zeros, J.nx, bx, nullptr, s, false, &p->rs)) return 1;
      CUDA_OK(launch_scale(bx, -1.0, J.nx * 384, s));
      break;
    default: /* -L0(x,x) + L0(0,x) */
      if (run_l0(c, J.d_x, J.d_x, J.nx, bx, nullptr, s, false, &p->rs) ||
          run_l0(c, p->zeros, J.d_x, J.nx, p->bt[j], nullptr, s, false, &p->rs))
        return 1;
      CUDA_OK(launch_scale(bx, -1.0, J.nx * 384, s));
      CUDA_OK(launch_axpy(bx, p->bt[j], 1.0, J.nx * 384, s));
      break;
    }
    CUDA_OK(launch_to_float2(bx, p->bx2[j], J.nx * 384, s));
  }
  return 0;
}

int plan_enqueue_kernels(kqed_batch_plan *p, const LaunchCfg &cfg, cudaStream_t s,
                         size_t units = 0)
{
  CUDA_OK(launch_lattice_batch(p->c->T, p->c->M, p->shared, p->d_jobs, (int)p->hj.size(),
                               units ? units : p->units, cfg, s,
                               p->precision == KQED_FP32_MIXED));
  return 0;
}

/* the tuner times the batch's first kTuneUnits units (8.4 M pairs) */
constexpr size_t kTuneUnits = (size_t)1 << 17;

int plan_enqueue(kqed_batch_plan *p, cudaStream_t s)
{
  const bool mixed = p->precision == KQED_FP32_MIXED;
  for (size_t j = 0; j < p->jobs.size(); j++) {
    const kqed_lattice_job &J = p->jobs[j];
    CUDA_OK(launch_build_columns(p->c->T, J.d_x, J.nx, const_cast<double *>(p->hj[j].col), s));
    if (mixed)
      CUDA_OK(launch_build_columns32(p->c->T, J.d_x, J.nx, const_cast<float *>(p->hj[j].col32), s));
    else
      CUDA_OK(launch_to_float2(p->hj[j].col, const_cast<float2 *>(p->hj[j].coldf),
                               J.nx * (size_t)p->c->T.nstpy * p->c->T.NK * kRow, s));
  }
  if (plan_enqueue_terms(p, s)) return 1;
  if (plan_enqueue_kernels(p, p->cfg, s)) return 1;
  for (size_t j = 0; j < p->jobs.size(); j++)
    CUDA_OK(launch_reduce_partials(p->hj[j].partial, p->jobs[j].nx, p->hj[j].tiles,
                                   p->jobs[j].d_sums, s));
  return 0;
}

/* time the two main kernels of the batch under cfg (best of two runs) */
int plan_time(kqed_batch_plan *p, const LaunchCfg &cfg, cudaStream_t s, double *ms)
{
  cudaEvent_t a, b;
  CUDA_OK(cudaEventCreate(&a));
  CUDA_OK(cudaEventCreate(&b));
  double best = 1e300;
  for (int rep = 0; rep < 2; rep++) {
    CUDA_OK(cudaEventRecord(a, s));
    if (plan_enqueue_kernels(p, cfg, s, std::min(p->units, kTuneUnits))) return 1;
    CUDA_OK(cudaEventRecord(b, s));
    CUDA_OK(cudaEventSynchronize(b));
    float t = 0;
    CUDA_OK(cudaEventElapsedTime(&t, a, b));
    best = std::min(best, (double)t);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = best;
  return 0;
}

/* launch-parameter sweep: assembly warps per block, assembly grid, record
   chunk; results kept per (device, precision, log2 of the batch's units) */
struct TuneKey { int dev, precision, lg; LaunchCfg cfg; size_t chunk; };
std::mutex g_tune_mu;
std::vector<TuneKey> g_tuned;

int plan_tune(kqed_batch_plan *p, cudaStream_t s)
{
  int dev = 0;
  cudaGetDevice(&dev);
  int lg = 0;
  for (size_t u = p->units; u > 1; u >>= 1) lg++;
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    for (const auto &t : g_tuned)
      if (t.dev == dev && t.precision == p->precision && t.lg == lg && t.chunk <= p->rs.cap) {
        p->cfg = t.cfg;
        p->shared.rec_cap = t.chunk;
        return 0;
      }
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t full = p->rs.cap;
  const size_t chunks[2] = {full, std::max((size_t)kTile, full / 4 / kTile * kTile)};
  double best = 1e300;
  LaunchCfg bc = p->cfg;
  size_t bchunk = full;
  for (int w : {2, 4})
    for (int bpsm : {0, 2, 1})
      for (size_t ch : chunks) {
        LaunchCfg cfg = p->cfg;
        cfg.warps_per_block = w;
        cfg.blocks = bpsm ? bpsm * sms : 0;
        p->shared.rec_cap = ch;
        double ms = 0;
        if (plan_time(p, cfg, s, &ms)) return 1;
        if (ms < best) { best = ms; bc = cfg; bchunk = ch; }
      }
  p->cfg = bc;
  p->shared.rec_cap = bchunk;
  p->tuned_ms = best;
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tuned.push_back({dev, p->precision, lg, bc, bchunk});
  return 0;
}

} // namespace

extern "C" void kqed_batch_plan_destroy(kqed_batch_plan *p)
{
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->cap) cudaStreamDestroy(p->cap);
  for (void *m : p->allocs) cudaFree(m);
  delete p;
}

extern "C" int kqed_batch_plan_create(const struct QED_kernel_temps *t, int njobs,
                                      const struct kqed_lattice_job *jobs, int precision,
                                      int tune, kqed_batch_plan **plan)
{
  if (!plan) return fail("null plan pointer");
  *plan = nullptr;
  Ctx *c = ctx_of(t);
  if (!c) return fail("tables not initialised");
  if (njobs <= 0 || !jobs) return fail("empty batch");
  if (check_variant_precision(0, precision)) return 1;
  std::unique_ptr<kqed_batch_plan> P(new kqed_batch_plan);
  kqed_batch_plan *p = P.get();
  p->c = c;
  p->precision = precision;
  p->cfg = c->cfg;
  p->jobs.assign(jobs, jobs + njobs);
  const bool mixed = precision == KQED_FP32_MIXED;
  const size_t per_x = (size_t)c->T.nstpy * c->T.NK * kRow;
  size_t zmax = 0, total_pairs = 0;
  for (int j = 0; j < njobs; j++) {
    const kqed_lattice_job &J = jobs[j];
    if (J.variant < 0 || J.variant > 3) return fail("job %d: variant %d not in 0..3", j, J.variant);
    if (J.nx == 0 || J.ny == 0) return fail("job %d: empty lattice", j);
    if (!J.d_x || !J.d_y || !J.d_sums) return fail("job %d: null buffer", j);
    zmax = std::max(zmax, std::max(J.nx, J.ny));
  }
  if (plan_alloc(p, &p->zeros, zmax * 4)) return 1;
  CUDA_OK(cudaMemset(p->zeros, 0, zmax * 4 * sizeof(double)));
  p->hj.resize(njobs);
  p->bx.assign(njobs, nullptr);
  p->bt.assign(njobs, nullptr);
  p->bx2.assign(njobs, nullptr);
  for (int j = 0; j < njobs; j++) {
    const kqed_lattice_job &J = jobs[j];
    LatticeArgs &A = p->hj[j];
    A = LatticeArgs{};
    A.x = J.d_x;
    A.y = J.d_y;
    A.nx = J.nx;
    A.ny = J.ny;
    A.pi = J.d_pi;
    A.pi_seed = J.pi_seed;
    A.pi_stream = J.pi_stream;
    A.k0 = 0;
    A.tiles = (int)((J.ny + kTile - 1) / kTile);
    A.u_begin = p->units;
    p->units += J.nx * (size_t)A.tiles;
    total_pairs += J.nx * (size_t)A.tiles * kTile;
    if (plan_alloc(p, &A.partial, J.nx * (size_t)A.tiles * 2)) return 1;
    double *col = nullptr;
    if (plan_alloc(p, &col, J.nx * per_x)) return 1;
    A.col = col;
    if (mixed) {
      float *c32 = nullptr;
      if (plan_alloc(p, &c32, J.nx * per_x)) return 1;
      A.col32 = c32;
    } else {
      float2 *cdf = nullptr;
      if (plan_alloc(p, &cdf, J.nx * per_x)) return 1;
      A.coldf = cdf;
    }
    if (J.variant) {
      /* per-site term, shared with earlier jobs on the same sites */
      const int kind = yterm_kind(J.variant);
      kqed_batch_plan::YTerm *Y = nullptr;
      for (auto &q : p->yterms)
        if (q.d_y == J.d_y && q.ny == J.ny && q.kind == kind) Y = &q;
      if (!Y) {
        p->yterms.push_back({J.d_y, J.ny, kind, nullptr, nullptr});
        Y = &p->yterms.back();
        if (plan_alloc(p, &Y->ky, J.ny * 384)) return 1;
        if (plan_alloc(p, &Y->ky2, J.ny * 384)) return 1;
      }
      A.Ky = Y->ky;
      A.Ky2 = Y->ky2;
      A.zero_x_vanishes = J.variant >= 2;
      if (plan_alloc(p, &p->bx[j], J.nx * 384)) return 1;
      if (J.variant == 3 && plan_alloc(p, &p->bt[j], J.nx * 384)) return 1;
      if (plan_alloc(p, &p->bx2[j], J.nx * 384)) return 1;
      A.Bx = p->bx[j];
      A.Bx2 = p->bx2[j];
    }
  }
  /* record space: the batch's kernels and the term launches share it; a
     plan owns its own, so it takes up to 16 M pairs (11 GB) -- at most an
     eighth of the free device memory -- and the captured graph holds 16x
     fewer record / assembly launch pairs than with the per-call chunk */
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const size_t per_pair = kRec * sizeof(double) + 12;
  const size_t plan_cap = std::max(kRecPairs, std::min((size_t)16 << 20, free_b / 8 / per_pair));
  size_t cap = std::min(std::max(total_pairs, zmax), plan_cap);
  cap = (cap + kTile - 1) / kTile * kTile;
  double *rb = nullptr;
  if (plan_alloc(p, &rb, cap * kRec + cap + cap / 2 + 1 + cap / 8 + 1)) return 1;
  p->rs = {rb, reinterpret_cast<uint8_t *>(rb + cap * kRec + cap + cap / 2 + 1), cap};
  p->shared = LatticeArgs{};
  p->shared.rec = rb;
  p->shared.env = rb + cap * kRec;
  p->shared.list = reinterpret_cast<uint32_t *>(rb + cap * kRec + cap);
  p->shared.count = reinterpret_cast<unsigned *>(rb + cap * kRec + cap + cap / 2);
  p->shared.code = p->rs.code;
  p->shared.rec_cap = cap;
  if (plan_alloc(p, &p->d_jobs, njobs)) return 1;
  CUDA_OK(cudaMemcpy(p->d_jobs, p->hj.data(), njobs * sizeof(LatticeArgs), cudaMemcpyHostToDevice));
  CUDA_OK(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking));
  /* eager run: sets every launch attribute, fills the tables, and (tune)
     times the candidate launch parameters on the real batch */
  if (plan_enqueue(p, p->cap)) return 1;
  if (tune && plan_tune(p, p->cap)) return 1;
  CUDA_OK(cudaStreamSynchronize(p->cap));
  /* capture */
  CUDA_OK(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
  const int rc = plan_enqueue(p, p->cap);
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(p->cap, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return 1;
  }
  CUDA_OK(ec);
  p->graph = g;
  CUDA_OK(cudaGraphInstantiate(&p->exec, p->graph, 0));
  size_t nodes = 0;
  CUDA_OK(cudaGraphGetNodes(p->graph, nullptr, &nodes));
  std::vector<cudaGraphNode_t> nv(nodes);
  CUDA_OK(cudaGraphGetNodes(p->graph, nv.data(), &nodes));
  for (auto n : nv) {
    cudaGraphNodeType ty;
    if (cudaGraphNodeGetType(n, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel)
      p->graph_kernels++;
  }
  *plan = P.release();
  return 0;
}

extern "C" int kqed_batch_plan_launch(kqed_batch_plan *p, void *stream)
{
  if (!p || !p->exec) return fail("invalid batch plan");
  CUDA_OK(cudaGraphLaunch(p->exec, (cudaStream_t)stream));
  g_launches += p->graph_kernels;
  return 0;
}

extern "C" int kqed_batch_plan_info(const kqed_batch_plan *p, struct kqed_batch_info *info)
{
  if (!p || !info) return fail("null argument");
  info->jobs = (int)p->jobs.size();
  info->units = p->units;
  info->pairs = 0;
  for (const auto &J : p->jobs) info->pairs += J.nx * J.ny;
  info->warps_per_block = p->cfg.warps_per_block;
  info->blocks = p->cfg.blocks;
  info->record_chunk_pairs = p->shared.rec_cap;
  info->graph_kernels = p->graph_kernels;
  info->tuned_ms = p->tuned_ms;
  return 0;
}
