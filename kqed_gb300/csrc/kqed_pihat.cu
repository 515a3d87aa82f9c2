/*
 * The perturbative lepton-loop Pi-hat on the GPU (src/LIBFILES/pi_pert.c of
 * the reference): ipihatFermLoop_antisym(x, y) -- the (rho, sigma)-
 * antisymmetrised four-point function of a free lepton loop in position
 * space, the Pi-hat that the QED kernel is contracted with for the
 * lepton-loop check of a_mu (src/amu_forlattice.c:65-116) -- batched over
 * pairs, in the lattice layout [nx][ny][384] of the fused lattice sums, and
 * per pair with the reference's signature; plus the reference's host
 * helpers of the same file (init_g8, diractrace, bessk, amu_heavlept,
 * amu_lightlept, vac_pol).
 *
 * One pihat1 call (pi_pert.c:236-389) is, for each of its 256 rows
 * r = (sigma, mu, nu, lambda), a sum over (alpha, beta, gamma, delta) of
 * G8[alpha,mu,beta,nu,gamma,sigma,delta,lambda] xab[alpha][beta] fv[gamma][delta][.]
 * plus dense terms with the six- and four-index traces.  G8 = 4 tr(8
 * gammas) is 0 or +-4 and non-zero at 8,320 of its 65,536 entries (24 to
 * 40 per row), so each row walks its own list of non-zero entries (in the
 * reference's (alpha, beta, gamma, delta) order, so that the sums round as
 * the reference's do: skipped terms add an exact zero).
 *
 * Kernel: persistent blocks of 256 threads, one thread per row; the block
 * holds the sparse G8 rows (17 KB), the six- and four-index traces, and per
 * pair the constants of the three pihat1 calls and their 3 x 1,280 outputs
 * in shared memory, then forms the 384 antisymmetrised components.  All
 * FP64, the reference's order of operations (no contraction into FMAs).
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/kqed.h"
#include "kqed_internal.h"

namespace kqed {
namespace {

/* 1/4 tr(gamma_{i0} ... gamma_{i(n-1)}), Euclidean: the last gamma is moved
   to the front through the anticommutators {gamma_a, gamma_b} = 2 delta_ab */
int trace_quarter(int n, const int *idx)
{
  if (n & 1) return 0;
  if (n == 0) return 1;
  if (n == 2) return idx[0] == idx[1];
  int red[16], acc = 0;
  for (int i = 0; i < n - 1; i++) {
    if (idx[i] != idx[n - 1]) continue;
    int k = 0;
    for (int j = 0; j < n - 1; j++)
      if (j != i) red[k++] = idx[j];
    acc += ((i & 1) ? -1 : 1) * trace_quarter(n - 2, red);
  }
  return acc;
}

void fill_g8(int *g8)
{
  for (int i = 0; i < 65536; i++) {
    int idx[8];
    for (int k = 0; k < 8; k++) idx[k] = (i >> (2 * (7 - k))) & 3;
    g8[i] = 4 * trace_quarter(8, idx);
  }
}

/* K_0 .. K_n at x > 0 (the polynomial approximations of Abramowitz &
   Stegun 9.8.5-9.8.8 for K_0, K_1 -- the ones pi_pert.c:95-137 uses -- and
   the recurrence K_{j+1} = K_{j-1} + (2j/x) K_j) */
__host__ __device__ inline void bessel_k(int n, double x, double *bv)
{
  double k0, k1;
  const double tox = 2.0 / x;
  if (x <= 2.0) {
    double t = x / 3.75;
    t *= t;
    const double i0 = 1.0 + t * (3.5156229 + t * (3.0899424 + t * (1.2067492 + t * (0.2659732 +
                      t * (0.360768e-1 + t * 0.45813e-2)))));
    const double i1 = x * (0.5 + t * (0.87890594 + t * (0.51498869 + t * (0.15084934 + t *
                      (0.2658733e-1 + t * (0.301532e-2 + t * 0.32411e-3))))));
    t = 0.25 * x * x;
    const double lg = log(x / 2.0);
    k0 = (-lg * i0) + (-0.57721566 + t * (0.42278420 + t * (0.23069756 + t * (0.3488590e-1 +
         t * (0.262698e-2 + t * (0.10750e-3 + t * 0.74e-5))))));
    k1 = (lg * i1) + (1.0 / x) * (1.0 + t * (0.15443144 + t * (-0.67278579 + t * (-0.18156897 +
         t * (-0.1919402e-1 + t * (-0.110404e-2 + t * (-0.4686e-4)))))));
  } else {
    const double e = exp(-x) / sqrt(x);
    k0 = e * (1.25331414 + tox * (-0.7832358e-1 + tox * (0.2189568e-1 + tox * (-0.1062446e-1 +
         tox * (0.587872e-2 + tox * (-0.251540e-2 + tox * 0.53208e-3))))));
    k1 = e * (1.25331414 + tox * (0.23498619 + tox * (-0.3655620e-1 + tox * (0.1504268e-1 +
         tox * (-0.780353e-2 + tox * (0.325614e-2 + tox * (-0.68245e-3)))))));
  }
  bv[0] = k0;
  if (n < 1) return;
  bv[1] = k1;
  double km = k0, k = k1;
  for (int j = 1; j < n; j++) {
    const double kp = km + j * tox * k;
    km = k;
    bv[j + 1] = k = kp;
  }
}

/* sparse G8 rows: entries (alpha, beta, gamma, delta) in 8 bits plus the
   sign, row r = sigma*64 + mu*16 + nu*4 + lambda */
constexpr int kG8Nz = 8320;
struct PihatTables {
  uint16_t *ent = nullptr;   /* [kG8Nz]: bits 0-7 (a<<6|b<<4|c<<2|d), bit 8 = negative */
  uint16_t *off = nullptr;   /* [257] */
  int8_t *g6 = nullptr;      /* [4096] = G8 with two leading zero indices, / 4 */
};

int build_tables(PihatTables &P)
{
  std::vector<int> g8(65536);
  fill_g8(g8.data());
  std::vector<uint16_t> ent, off(257);
  for (int r = 0; r < 256; r++) {
    off[r] = (uint16_t)ent.size();
    const int sig = r >> 6, mu = (r >> 4) & 3, nu = (r >> 2) & 3, la = r & 3;
    for (int ab = 0; ab < 16; ab++)
      for (int cd = 0; cd < 16; cd++) {
        const int a = ab >> 2, b = ab & 3, c = cd >> 2, d = cd & 3;
        const int v = g8[((((((a * 4 + mu) * 4 + b) * 4 + nu) * 4 + c) * 4 + sig) * 4 + d) * 4 + la];
        if (v == 0) continue;
        if (v != 4 && v != -4) return set_error("pihat: unexpected Dirac-trace value");
        ent.push_back((uint16_t)((ab << 4) | cd | (v < 0 ? 256 : 0)));
      }
  }
  off[256] = (uint16_t)ent.size();
  if ((int)ent.size() != kG8Nz) return set_error("pihat: unexpected Dirac-trace sparsity");
  std::vector<int8_t> g6(4096);
  for (int i = 0; i < 4096; i++) g6[i] = (int8_t)(g8[i] / 4);
  if (cudaMalloc(&P.ent, kG8Nz * sizeof(uint16_t)) != cudaSuccess ||
      cudaMalloc(&P.off, 257 * sizeof(uint16_t)) != cudaSuccess ||
      cudaMalloc(&P.g6, 4096) != cudaSuccess)
    return set_error("pihat: out of device memory for the trace tables");
  if (cudaMemcpy(P.ent, ent.data(), kG8Nz * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(P.off, off.data(), 257 * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(P.g6, g6.data(), 4096, cudaMemcpyHostToDevice) != cudaSuccess)
    return set_error("pihat: upload of the trace tables failed");
  return 0;
}

/* the device's tables, built on first use (never freed: 42 KB per device) */
int tables_for_device(PihatTables *out)
{
  static std::mutex mu;
  static PihatTables per[64];
  static bool ready[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return set_error("pihat: no CUDA device");
  std::lock_guard<std::mutex> lk(mu);
  if (!ready[dev]) {
    if (build_tables(per[dev])) return 1;
    ready[dev] = true;
  }
  *out = per[dev];
  return 0;
}

/* per pihat1 call, the pair constants (pi_pert.c:243-331) */
struct CallC {
  double xv[4], g[4], q[4], x2[4], x3[4];
  double xab[4][4], ht[4][4], fhat[4][4], ell[4][4];
  double fv[4][4][4];
  double p, b11, nrm;
};

__device__ void call_constants(const double *x, const double *y, CallC &C)
{
  const double pp = M_PI * M_PI, tpp = 2 * pp;
  double xmy[4];
  for (int r = 0; r < 4; r++) xmy[r] = __dsub_rn(x[r], y[r]);
  auto nrm4 = [](const double *v) {
    return sqrt(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])),
                                    __dmul_rn(v[2], v[2])),
                          __dmul_rn(v[3], v[3])));
  };
  const double xn = nrm4(x), yn = nrm4(y), dn = nrm4(xmy);
  double bx[3], by[3], bd[3];
  bessel_k(2, xn, bx);
  bx[1] = __ddiv_rn(bx[1], xn);
  bx[2] = __ddiv_rn(bx[2], __dmul_rn(xn, xn));
  bessel_k(2, yn, by);
  by[1] = __ddiv_rn(by[1], yn);
  by[2] = __ddiv_rn(by[2], __dmul_rn(yn, yn));
  bessel_k(2, dn, bd);
  bd[1] = __ddiv_rn(bd[1], dn);
  bd[2] = __ddiv_rn(bd[2], __dmul_rn(dn, dn));
  double e[4], f[4];
  for (int r = 0; r < 4; r++) {
    C.xv[r] = x[r];
    e[r] = __dmul_rn(__dmul_rn(tpp, y[r]), by[2]);
    f[r] = __dmul_rn(__dmul_rn(pp, y[r]), by[1]);
    C.g[r] = __dmul_rn(__dmul_rn(pp, y[r]), by[0]);
    C.q[r] = __dmul_rn(2.0, f[r]);
  }
  C.p = __dmul_rn(tpp, by[0]);
  const double s = __dmul_rn(tpp, by[1]);
  double h[4][4];
  for (int r = 0; r < 4; r++)
    for (int d = 0; d < 4; d++) {
      h[r][d] = __dmul_rn(f[r], y[d]);
      C.ell[r][d] = __dmul_rn(e[r], y[d]);
      if (r == d) {
        h[r][d] = __dsub_rn(h[r][d], __dmul_rn(0.5, C.p));
        C.ell[r][d] = __dsub_rn(C.ell[r][d], s);
      }
    }
  for (int r = 0; r < 4; r++)
    for (int d = 0; d < 4; d++) {
      C.ht[r][d] = h[d][r];
      C.fhat[d][r] = h[r][d];
    }
  for (int r = 0; r < 4; r++) {
    for (int d = 0; d < 4; d++)
      for (int c = 0; c < 4; c++) {
        const double cube = __dmul_rn(__dmul_rn(__dmul_rn(by[2], y[c]), y[d]), y[r]);
        const double lin = __dsub_rn(__dsub_rn(__dmul_rn((double)(r == d), y[c]),
                                               __dmul_rn((double)(c == r), y[d])),
                                     __dmul_rn((double)(c == d), y[r]));
        C.fv[c][d][r] = __dmul_rn(pp, __dadd_rn(cube, __dmul_rn(lin, by[1])));
      }
    C.fhat[r][r] = __dadd_rn(C.fhat[r][r], C.p);
  }
  C.b11 = __dmul_rn(bx[1], bd[1]);
  const double b12 = __dmul_rn(bx[1], bd[2]), b21 = __dmul_rn(bx[2], bd[1]),
               b22 = __dmul_rn(bx[2], bd[2]);
  for (int a = 0; a < 4; a++) {
    for (int b = 0; b < 4; b++) C.xab[a][b] = __dmul_rn(__dmul_rn(x[a], xmy[b]), b22);
    C.x2[a] = __dmul_rn(x[a], b21);
    C.x3[a] = __dmul_rn(xmy[a], b12);
  }
  C.nrm = 8.2336243479292e-07; /* 2 / (2 pi)^8 */
}

/* one pihat1 row: P[rho] (4) and R of row (sig, mu, nu, la) */
__device__ void pihat_row(const CallC &C, const uint16_t *ent, const uint16_t *off,
                          const int8_t *g6, int row, double P[4], double &R)
{
  const int sig = row >> 6, mu = (row >> 4) & 3, nu = (row >> 2) & 3, la = row & 3;
  auto G6 = [&](int c, int d, int e, int f, int g, int h) {
    return (double)(4 * g6[((((c * 4 + d) * 4 + e) * 4 + f) * 4 + g) * 4 + h]);
  };
  double t1[4] = {0.0, 0.0, 0.0, 0.0}, tr1 = 0.0;
  int k = off[row];
  const int kend = off[row + 1];
  for (int ab = 0; ab < 16; ab++) {
    const int a = ab >> 2, b = ab & 3;
    const double xab = C.xab[a][b];
    for (; k < kend && (ent[k] >> 4 & 15) == ab; k++) {
      const int e = ent[k], c = (e >> 2) & 3, d = e & 3;
      const double T = __dmul_rn(xab, (e & 256) ? -4.0 : 4.0);
#pragma unroll
      for (int r = 0; r < 4; r++) t1[r] = __dsub_rn(t1[r], __dmul_rn(C.fv[c][d][r], T));
      tr1 = __dsub_rn(tr1, __dmul_rn(C.ell[c][d], T));
    }
    const double m1 = __dmul_rn(G6(a, mu, b, nu, sig, la), xab);
    const double m2 = __dsub_rn(__dmul_rn(G6(a, mu, nu, b, sig, la), C.x2[a]),
                                __dmul_rn(G6(mu, a, nu, b, sig, la), C.x3[a]));
    const double m4 = __dsub_rn(__dmul_rn(G6(a, mu, nu, sig, b, la), C.x2[a]),
                                __dmul_rn(G6(mu, a, nu, sig, b, la), C.x3[a]));
    const double m6 = __dmul_rn(G6(mu, nu, a, sig, b, la), C.b11);
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const double u = __dadd_rn(__dsub_rn(__dsub_rn(__dmul_rn(-C.g[r], m1), __dmul_rn(C.ht[b][r], m2)),
                                           __dmul_rn(C.fhat[b][r], m4)),
                                 __dmul_rn(C.fv[a][b][r], m6));
      t1[r] = __dadd_rn(t1[r], u);
    }
    tr1 = __dsub_rn(tr1, __dmul_rn(C.p, m1));
    tr1 = __dsub_rn(tr1, __dmul_rn(C.q[b], __dadd_rn(m2, m4)));
    tr1 = __dadd_rn(tr1, __dmul_rn(C.ell[a][b], m6));
  }
  const double m = __dmul_rn(G6(0, 0, mu, nu, sig, la), C.b11);
#pragma unroll
  for (int r = 0; r < 4; r++) P[r] = __dmul_rn(C.nrm, __dadd_rn(t1[r], __dmul_rn(C.g[r], m)));
  R = __dmul_rn(C.nrm, __dadd_rn(tr1, __dmul_rn(C.p, m)));
}

enum PihatMode { kPairs = 0, kLattice = 1, kRaw = 2 };

struct PihatArgs {
  PihatTables tab;
  const double *x, *y;
  size_t n, nx, ny; /* kPairs / kRaw: n pairs; kLattice: nx * ny pairs (k-major) */
  double scale;     /* kLattice: arguments scale * x_k, scale * y_n */
  double *out;
  int mode;
};

constexpr int kPiThreads = 256;

struct PiSmem {
  uint16_t ent[kG8Nz];
  uint16_t off[257];
  int8_t g6[4096];
  CallC C[3];
  double P[3][4][256]; /* [call][rho][row = mu*64+nu*16+la*4+sig ordering below] */
  double R[3][256];
};

__global__ void __launch_bounds__(kPiThreads) pihat_kernel(const __grid_constant__ PihatArgs A)
{
  extern __shared__ __align__(16) unsigned char smraw[];
  PiSmem &S = *reinterpret_cast<PiSmem *>(smraw);
  const int tid = threadIdx.x;
  for (int i = tid; i < kG8Nz; i += kPiThreads) S.ent[i] = A.tab.ent[i];
  for (int i = tid; i < 257; i += kPiThreads) S.off[i] = A.tab.off[i];
  for (int i = tid; i < 4096; i += kPiThreads) S.g6[i] = A.tab.g6[i];
  const size_t total = A.mode == kLattice ? A.nx * A.ny : A.n;
  for (size_t pr = blockIdx.x; pr < total; pr += gridDim.x) {
    double xv[4], yv[4];
    if (A.mode == kLattice) {
      const size_t k = pr / A.ny, n = pr % A.ny;
      for (int m = 0; m < 4; m++) {
        xv[m] = __dmul_rn(A.scale, A.x[4 * k + m]);
        yv[m] = __dmul_rn(A.scale, A.y[4 * n + m]);
      }
    } else {
      for (int m = 0; m < 4; m++) { xv[m] = A.x[4 * pr + m]; yv[m] = A.y[4 * pr + m]; }
    }
    __syncthreads(); /* tables loaded / previous pair's outputs consumed */
    if (tid < 3 && (A.mode != kRaw || tid == 0)) {
      /* the three photon orderings of ipihatFermLoop_antisym (pi_pert.c:168-176):
         (x, y), (y - x, -x), (-x, y - x) */
      double a[4], b[4];
      for (int m = 0; m < 4; m++) {
        const double mx = -xv[m], ymx = __dsub_rn(yv[m], xv[m]);
        a[m] = tid == 0 ? xv[m] : (tid == 1 ? ymx : mx);
        b[m] = tid == 0 ? yv[m] : (tid == 1 ? mx : ymx);
      }
      call_constants(a, b, S.C[tid]);
    }
    __syncthreads();
    const int ncall = A.mode == kRaw ? 1 : 3;
    for (int c = 0; c < ncall; c++) {
      double P[4], R;
      pihat_row(S.C[c], S.ent, S.off, S.g6, tid, P, R);
      /* stored as the reference's vpihat1[rho][mu][nu][la][sig] */
      const int sig = tid >> 6, mu = (tid >> 4) & 3, nu = (tid >> 2) & 3, la = tid & 3;
      const int o = mu * 64 + nu * 16 + la * 4 + sig;
#pragma unroll
      for (int r = 0; r < 4; r++) S.P[c][r][o] = P[r];
      S.R[c][o] = R;
    }
    __syncthreads();
    if (A.mode == kRaw) {
      double *o = A.out + pr * 1280;
      for (int i = tid; i < 1024; i += kPiThreads) o[i] = S.P[0][i >> 8][i & 255];
      o[1024 + tid] = S.R[0][tid];
      continue;
    }
    double *o = A.out + pr * 384;
    for (int i = tid; i < 384; i += kPiThreads) {
      const int rs = i >> 6, mu = (i >> 4) & 3, nu = (i >> 2) & 3, la = i & 3;
      const int rho = rs < 3 ? 0 : (rs < 5 ? 1 : 2);
      const int sig = rs < 3 ? rs + 1 : (rs < 5 ? rs - 1 : 3);
      auto P = [&](int c, int r, int b, int cc, int d, int e) {
        return S.P[c][r][b * 64 + cc * 16 + d * 4 + e];
      };
      auto R = [&](int c, int b, int cc, int d, int e) { return S.R[c][b * 64 + cc * 16 + d * 4 + e]; };
      double u = __dadd_rn(P(0, rho, mu, nu, la, sig), P(1, rho, nu, la, mu, sig));
      u = __dadd_rn(u, __dmul_rn(xv[rho], R(1, nu, la, mu, sig)));
      u = __dadd_rn(u, P(2, rho, la, nu, mu, sig));
      u = __dadd_rn(u, __dmul_rn(xv[rho], R(2, la, nu, mu, sig)));
      double w = __dadd_rn(P(0, sig, mu, nu, la, rho), P(1, sig, nu, la, mu, rho));
      w = __dadd_rn(w, __dmul_rn(xv[sig], R(1, nu, la, mu, rho)));
      w = __dadd_rn(w, P(2, sig, la, nu, mu, rho));
      w = __dadd_rn(w, __dmul_rn(xv[sig], R(2, la, nu, mu, rho)));
      o[i] = __dmul_rn(0.5, __dsub_rn(u, w));
    }
  }
}

int launch_pihat(PihatArgs A, cudaStream_t s)
{
  if (tables_for_device(&A.tab)) return 1;
  const size_t total = A.mode == kLattice ? A.nx * A.ny : A.n;
  if (total == 0) return 0;
  int dev = 0, sms = 0, per = 0;
  const size_t smem = sizeof(PiSmem);
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaFuncSetAttribute(pihat_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pihat_kernel, kPiThreads, smem) !=
          cudaSuccess)
    return set_error("pihat: launch configuration failed");
  const size_t grid = std::min(total, (size_t)std::max(per, 1) * sms);
  pihat_kernel<<<(unsigned)grid, kPiThreads, smem, s>>>(A);
  if (cudaGetLastError() != cudaSuccess) return set_error("pihat: launch failed");
  g_launches++;
  return 0;
}

int pihat_host(size_t n, const double *x, const double *y, double *out, int mode, size_t per_pair)
{
  if (n == 0) return 0;
  if (!x || !y || !out) return set_error("null buffer");
  double *d = nullptr;
  const size_t bytes = n * (8 + per_pair) * sizeof(double);
  if (cudaMalloc(&d, bytes) != cudaSuccess) return set_error("pihat: out of device memory");
  PihatArgs A{};
  A.x = d;
  A.y = d + 4 * n;
  A.out = d + 8 * n;
  A.n = n;
  A.mode = mode;
  int rc = 0;
  if (cudaMemcpy(d, x, n * 4 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d + 4 * n, y, n * 4 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    rc = set_error("pihat: copy to the device failed");
  if (!rc) rc = launch_pihat(A, nullptr);
  if (!rc && (cudaMemcpy(out, A.out, n * per_pair * sizeof(double), cudaMemcpyDeviceToHost) !=
              cudaSuccess))
    rc = set_error("pihat: execution or copy back failed");
  cudaFree(d);
  return rc;
}

} // namespace
} // namespace kqed

/* ------------------------------------------------------------- C ABI */

extern "C" int kqed_pihat_batch_dev(size_t n, const double *d_x, const double *d_y,
                                    double *d_out, void *stream)
{
  if (n && (!d_x || !d_y || !d_out)) return kqed::set_error("null buffer");
  kqed::PihatArgs A{};
  A.x = d_x;
  A.y = d_y;
  A.out = d_out;
  A.n = n;
  A.mode = kqed::kPairs;
  return kqed::launch_pihat(A, (cudaStream_t)stream);
}

extern "C" int kqed_pihat_batch(size_t n, const double *x, const double *y, double *out)
{
  return kqed::pihat_host(n, x, y, out, kqed::kPairs, 384);
}

extern "C" int kqed_pihat_lattice_dev(size_t nx, const double *d_x, size_t ny, const double *d_y,
                                      double scale, double *d_pi, void *stream)
{
  if (nx && ny && (!d_x || !d_y || !d_pi)) return kqed::set_error("null buffer");
  kqed::PihatArgs A{};
  A.x = d_x;
  A.y = d_y;
  A.out = d_pi;
  A.nx = nx;
  A.ny = ny;
  A.scale = scale;
  A.mode = kqed::kLattice;
  return kqed::launch_pihat(A, (cudaStream_t)stream);
}

extern "C" void ipihatFermLoop_antisym(const double x[4], const double y[4],
                                       const struct QED_kernel_temps t, double vpihat[6][4][4][4])
{
  (void)t;
  if (kqed::pihat_host(1, x, y, &vpihat[0][0][0][0], kqed::kPairs, 384)) {
    fprintf(stderr, "ipihatFermLoop_antisym: %s\n", kqed_last_error());
    memset(vpihat, 0, 384 * sizeof(double));
  }
}

extern "C" void pihat1(const double x[4], const double y[4], const struct QED_kernel_temps t,
                       double vpihat1[4][4][4][4][4], double vpihatr1[4][4][4][4])
{
  (void)t;
  double buf[1280];
  if (kqed::pihat_host(1, x, y, buf, kqed::kRaw, 1280)) {
    fprintf(stderr, "pihat1: %s\n", kqed_last_error());
    memset(buf, 0, sizeof(buf));
  }
  memcpy(&vpihat1[0][0][0][0][0], buf, 1024 * sizeof(double));
  memcpy(&vpihatr1[0][0][0][0], buf + 1024, 256 * sizeof(double));
}

extern "C" int diractrace(const int n, const int *idx)
{
  if (n < 0 || n > 16 || (n && !idx)) return 0;
  return kqed::trace_quarter(n, idx);
}

extern "C" void init_g8(struct QED_kernel_temps *t)
{
  if (t && t->G8) kqed::fill_g8(t->G8);
}

extern "C" void bessk(const int n, const double x, double *bv)
{
  kqed::bessel_k(n, x, bv);
}

/* The analytic lepton-loop results the lattice integration is checked
   against (the reference's pi_pert.c:49-92 and :391-404): the light-by-light
   contribution of a heavy lepton (mass ratio mh to the muon) and of a light
   lepton (ml), expansions of Laporta & Remiddi, Phys. Lett. B 301 (1993)
   440, Eqs. (4) and (2), including (alpha/pi)^3; and the two-loop vacuum
   polarisation term.  Unlike the reference, nothing is printed. */
namespace {
constexpr double kZeta3 = 1.2020569031595942854;
constexpr double kAlpha = 1.0 / 137.035999;
constexpr double kPi = 3.14159265358979323846;
}

extern "C" double amu_heavlept(const double mh)
{
  const double p2 = kPi * kPi, z2 = p2 / 6, m2 = mh * mh, m4 = m2 * m2, L = log(mh);
  const double c2 = (1.5 * kZeta3 - 19.0 / 16) / m2;
  const double c4 = (-161.0 / 810 * L * L - 16189.0 / 48600 * L + 13.0 / 18 * kZeta3 -
                     161.0 / 9720 * p2 - 831931.0 / 972000) / (m2 * m2);
  const double c6 = (17.0 / 36 * kZeta3 - 13.0 / 224 * z2 - 1840256147.0 / 3556224000 -
                     4381.0 / 120960 * 4.0 * L * L - 24761.0 / 317520 * 2.0 * L) / (m4 * m2);
  const double c8 = (7.0 / 20 * kZeta3 - 2047.0 / 54000 * z2 - 453410778211.0 / 1200225600000 -
                     5207.0 / 189000 * 4.0 * L * L - 41940853.0 / 952560000 * 2.0 * L) / (m4 * m4);
  const double c10 = (5.0 / 18 * kZeta3 - 1187.0 / 44550 * z2 - 86251554753071.0 / 287550049248000 -
                      328337.0 / 14968800 * 4.0 * L * L - 640572781.0 / 23051952000 * 2.0 * L) /
                     (m4 * m4 * m2);
  return kAlpha * kAlpha * kAlpha / (kPi * kPi * kPi) * (c2 + c4 + c6 + c8 + c10);
}

extern "C" double amu_lightlept(const double ml)
{
  const double p2 = kPi * kPi, p4 = p2 * p2, m2 = ml * ml, L = -log(ml), l2 = log(2.0);
  const double c1 = 2.0 / 3 * p2 * L;
  const double c2 = 59.0 / 270 * p4 - 3.0 * kZeta3 - 10.0 / 3 * p2 + 2.0 / 3;
  const double c3 = ml * (4.0 / 3 * p2 * L - 196.0 / 3 * p2 * l2 + 424.0 / 9 * p2);
  const double c4 = m2 * (-2.0 / 3 * L * L * L + (p2 / 9 - 20.0 / 3) * L * L -
                          (16.0 / 135 * p4 + 4.0 * kZeta3 - 32.0 / 9 * p2 + 61.0 / 3) * L +
                          4.0 / 3 * kZeta3 * p2 - 61.0 / 270 * p4 + 3.0 * kZeta3 + 25.0 / 18 * p2 -
                          283.0 / 12);
  const double c5 = m2 * ml * (10.0 / 9 * p2 * L - 11.0 / 9 * p2);
  const double c6 = m2 * m2 * (7.0 / 9 * L * L * L + 41.0 / 18 * L * L + 13.0 / 9 * p2 * L +
                               517.0 / 108 * L + kZeta3 / 2 + 191.0 / 216 * p2 + 13283.0 / 2592);
  return kAlpha * kAlpha * kAlpha / (kPi * kPi * kPi) * (c1 + c2 + c3 + c4 + c5 + c6);
}

extern "C" double vac_pol(const double ml)
{
  const double a4 = 0.51747906167389938633; /* Li_4(1/2) */
  const double p2 = kPi * kPi, m2 = ml * ml, L = -log(ml), l2 = log(2.0);
  const double c1 = 2.0 / 9 * L * L;
  const double c2 = (kZeta3 - 2.0 / 3 * p2 * l2 + p2 / 9 + 31.0 / 27) * L;
  const double c3 = 11.0 / 216 * p2 * p2 - 2.0 / 9 * p2 * l2 * l2 - 8.0 / 3 * a4 -
                    1.0 / 9 * l2 * l2 * l2 * l2 - 3.0 * kZeta3 + 5.0 / 3 * p2 * l2 -
                    25.0 / 18 * p2 + 1075.0 / 216;
  const double c4 = ml * (-13.0 / 18 * p2 * kPi - 16.0 / 9 * p2 * l2 + 3199.0 / 1080 * p2);
  const double c5 = m2 * (10.0 / 3 * L * L - 11.0 / 9 * L - 14.0 / 3 * p2 * l2 - 2.0 * kZeta3 +
                          49.0 / 12 * p2 - 131.0 / 54);
  const double c6 = ml * m2 * (4.0 / 3 * p2 * L + 35.0 / 12 * p2 * kPi - 16.0 / 3 * p2 * l2 -
                               5771.0 / 1080 * p2);
  return c1 + c2 + c3 + c4 + c5 + c6;
}
