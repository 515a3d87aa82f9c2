/*
 * Composite kernels on the GPU: the reference's linear combinations of L0
 * at derived arguments, with index permutations and Gaussian
 * M-subtractions --
 *   compute_all_kernels, compute_all_Mkernels(_v2)    src/LIBFILES/all_kernels.c:85-370
 *   compute_con_kernels(_v2), compute_con_kernelsM_L2 src/LIBFILES/con_kernel.c:61-399
 *   compute_sub_kernelsM_L2                           src/LIBFILES/sub_kernel.c:27-167
 *   compute_all_kernels_SYMXY(_v2)                    src/LIBFILES/SYMXY.c:14-85
 *   compute_all_kernels_SYMXY0(_v2)                   src/LIBFILES/SYMXY0.c:22-211
 *   QED_Mkernel_L2                                    src/LIBFILES/kernels.c:181-231
 * -- as one batched path for any number of pairs.
 *
 * Each composite is a small program: a list of derived L0 arguments (the
 * "sources": (x,y), (y,x), (x,0), (0,x-y), ...) and a list of slots, each a
 * sum of terms over earlier slots read at a permuted index, optionally with
 * the Gaussian subtraction e * (K - M u_a sum_alpha w_alpha K[..alpha..]),
 * then divided by a constant.  Slots either land in the output struct or
 * stay intermediate.  A batch of n pairs runs as
 *   1. derive_kernel: the sources' argument vectors, source-major ([j][i]),
 *      so that the L0 launch sees runs of one branch (the x = 0 / y = 0
 *      forms together) and its warps stay branch-uniform;
 *   2. one L0 batch over nsrc * n pairs (the library's record + assembly
 *      kernels, FP64 or mixed form);
 *   3. combine_kernel: one block per pair, one thread per component
 *      (rs, mu, nu, lambda); the pair's sources are staged in shared memory,
 *      every slot is evaluated in FP64 -- in the FP64 form in the
 *      reference's order of operations (no contraction into FMAs), in the
 *      mixed form with each Gaussian term as two fused multiply-adds (half
 *      the FP64 operations; this kernel is FP64-pipe-bound on GB300) --
 *      and outputs are written coalesced in the reference's struct layout.
 * The programs are written out below, term by term from the reference
 * functions they replace; the kernels are generic over them.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <initializer_list>
#include <mutex>
#include <vector>

#include "../../include/kqed.h"
#include "kqed_internal.h"

namespace kqed {
namespace {

/* derived argument vectors */
enum Arg : int8_t { AZ = 0, AX, AY, AXMY, AYMX, AMY };
/* vectors of the Gaussian terms */
enum Vec : int8_t { VN = 0, VX = 1, VY = 2, VXMY = 3 };
/* Gaussian factors exp(-M |v|^2 / 2) */
enum Gau : int8_t { G1 = 0, GX = 1, GY = 2, GXMY = 3 };

/* a slot or source read at [rs][o[p0]][o[p1]][o[p2]], o = (mu, nu, lambda) */
struct Perm {
  uint8_t a, b, c;
};
constexpr Perm I{0, 1, 2};   /* [mu][nu][la] */
constexpr Perm NML{1, 0, 2}; /* [nu][mu][la] */
constexpr Perm LNM{2, 1, 0}; /* [la][nu][mu] */
constexpr Perm LMN{2, 0, 1}; /* [la][mu][nu] */
constexpr Perm MLN{0, 2, 1}; /* [mu][la][nu] */
constexpr Perm NLM{1, 2, 0}; /* [nu][la][mu] */

/* coef * S[perm]                                  (g == G1), or
   (coef * e_g[mass]) * (S[perm] - (M[mass] * u[o[uslot]]) * pf),
   pf = sum_alpha w[alpha] S[perm with source position wpos = alpha]; pf
   comes from contraction table ct (one per distinct (src, wpos, w)) */
struct CTerm {
  uint8_t src, p0, p1, p2;
  int8_t g, mass, u, uslot, w, wpos, ct;
  int8_t pad;
  double coef;
};
/* contraction table: T[rs][a][b] = sum_alpha w[alpha] S_src[rs][..alpha..]
   with alpha at source position wpos and (a, b) the other two positions */
struct CCon {
  int8_t src, wpos, w, pad;
};
struct CSlot {
  uint16_t first, count;
  int16_t out; /* component block of the output struct, -1: intermediate */
  int16_t pad;
  double div;  /* 1: none */
};

constexpr int kMaxSrc = 12, kMaxSlot = 24, kMaxTerm = 112, kMaxCon = 8, kComp = 384;
constexpr int kConLen = 96; /* 6 x 4 x 4 */

struct CProgram {
  int nsrc, nslot, nout, ncon, nterm;
  int8_t a[kMaxSrc], b[kMaxSrc];
  double M[4];
  CCon con[kMaxCon];
  CSlot slot[kMaxSlot];
  CTerm term[kMaxTerm];
};

/* ------------------------------------------------------------ builder */

struct PB {
  CProgram p;
  int nterm = 0;
  bool bad = false;
  PB() { memset(&p, 0, sizeof(p)); }
  int src(Arg a, Arg b)
  {
    if (p.nslot) bad = true; /* sources come first */
    if (p.nsrc >= kMaxSrc) { bad = true; return 0; }
    p.a[p.nsrc] = a;
    p.b[p.nsrc] = b;
    return p.nsrc++;
  }
  int slot(int out, double div, std::initializer_list<CTerm> ts)
  {
    if (p.nslot >= kMaxSlot || nterm + (int)ts.size() > kMaxTerm) { bad = true; return 0; }
    CSlot &s = p.slot[p.nslot];
    s.first = (uint16_t)nterm;
    s.count = (uint16_t)ts.size();
    s.out = (int16_t)out;
    s.div = div;
    for (CTerm t : ts) {
      if (t.src >= p.nsrc + p.nslot) bad = true; /* only earlier slots */
      if (t.g != 0) {
        int c = 0;
        while (c < p.ncon && !(p.con[c].src == t.src && p.con[c].wpos == t.wpos &&
                               p.con[c].w == t.w))
          c++;
        if (c == p.ncon) {
          if (p.ncon >= kMaxCon) { bad = true; c = 0; }
          else p.con[p.ncon++] = CCon{(int8_t)t.src, t.wpos, t.w, 0};
        }
        t.ct = (int8_t)c;
      }
      p.term[nterm++] = t;
    }
    p.nterm = nterm;
    if (out >= 0) p.nout = std::max(p.nout, out + 1);
    return p.nsrc + p.nslot++;
  }
};

CTerm T(int s, Perm q = I, double coef = 1.0)
{
  CTerm t{};
  t.src = (uint8_t)s;
  t.p0 = q.a; t.p1 = q.b; t.p2 = q.c;
  t.coef = coef;
  return t;
}

/* Gaussian term: coef * e_g[mass] * (S[q] - M[mass] u[o[us]] sum_alpha w_alpha S[q, wp = alpha]) */
CTerm G(int s, Perm q, double coef, Gau g, int mass, Vec u, int us, Vec w, int wp)
{
  CTerm t = T(s, q, coef);
  t.g = g; t.mass = (int8_t)mass; t.u = u; t.uslot = (int8_t)us; t.w = w; t.wpos = (int8_t)wp;
  return t;
}

constexpr int MU = 0, NU = 1, LA = 2;

/* compute_all_kernels, all_kernels.c:85-166.  Returns the slots of
   L0.xy, L0.yx, L1.xy, L1.yx, ..., L3.yx; `outputs` false keeps them
   intermediate (the SYMXY forms). */
void prog_all_slots(PB &P, bool outputs, int W[8])
{
  const int sxy = P.src(AX, AY), syx = P.src(AY, AX), sx0 = P.src(AX, AZ), s0x = P.src(AZ, AX),
            sy0 = P.src(AY, AZ), s0y = P.src(AZ, AY);
  auto o = [&](int k) { return outputs ? k : -1; };
  const int f1 = P.slot(-1, 2.0, {T(sx0, LNM), T(sy0, LNM)});
  const int f2 = P.slot(-1, 1.0, {T(sx0), T(s0y)});
  const int f4 = P.slot(-1, 1.0, {T(s0x), T(sy0)});
  const int f3 = P.slot(-1, 1.0, {T(s0x), T(s0y, I, -1)});
  W[0] = P.slot(o(0), 1.0, {T(sxy)});
  W[1] = P.slot(o(1), 1.0, {T(syx)});
  W[2] = P.slot(o(2), 1.0, {T(sxy), T(f1)});
  W[4] = P.slot(o(4), 1.0, {T(sxy), T(f2, I, -1)});
  W[6] = P.slot(o(6), 1.0, {T(sxy), T(sx0, LNM), T(f3)});
  W[3] = P.slot(o(3), 1.0, {T(syx), T(f1)});
  W[5] = P.slot(o(5), 1.0, {T(syx), T(f4, I, -1)});
  W[7] = P.slot(o(7), 1.0, {T(syx), T(sy0, LNM), T(f3, I, -1)});
}

/* compute_all_Mkernels (all_kernels.c:211-286) and _v2 (:290-370) */
void prog_all_M(PB &P, bool v2)
{
  const int sxy = P.src(AX, AY);
  const int sxmy = v2 ? P.src(AX, AMY) : -1;
  const int syx = P.src(AY, AX), sx0 = P.src(AX, AZ), s0x = P.src(AZ, AX), sy0 = P.src(AY, AZ),
            s0y = P.src(AZ, AY);
  for (int a = 0; a < 4; a++) {
    /* inlineXY(a) */
    const int XY = P.slot(-1, 1.0, {G(s0y, I, 1, GX, a, VX, MU, VX, 0),
                                    G(sx0, I, 1, GY, a, VY, NU, VY, 1)});
    if (!v2) {
      /* inlineYX(a) */
      const int YX = P.slot(-1, 1.0, {G(s0x, I, 1, GY, a, VY, MU, VY, 0),
                                      G(sy0, I, 1, GX, a, VX, NU, VX, 1)});
      P.slot(2 * a, 1.0, {T(sxy), T(XY, I, -1)});
      P.slot(2 * a + 1, 1.0, {T(syx), T(YX, I, -1)});
    } else {
      /* inlineYX2(a), inlineXMY(a) */
      const int YX2 = P.slot(-1, 1.0, {G(s0x, NML, 1, GY, a, VY, NU, VY, 0),
                                       G(sy0, NML, 1, GX, a, VX, MU, VX, 1)});
      const int XMY = P.slot(-1, 1.0, {G(s0y, I, -1, GX, a, VX, MU, VX, 0),
                                       G(sx0, I, 1, GY, a, VY, NU, VY, 1)});
      P.slot(2 * a, 1.0, {T(sxy), T(XY, I, -1), T(syx, NML), T(YX2, I, -1)});
      P.slot(2 * a + 1, 1.0, {T(sxmy), T(XMY, I, -1)});
    }
  }
}

struct ConSrc {
  int xy, yx, xxmy, x0, s0x, y0, s0y, xmy0, s0xmy;
};
ConSrc con_sources(PB &P, bool with_xmy0)
{
  ConSrc s;
  s.xy = P.src(AX, AY);
  s.yx = P.src(AY, AX);
  s.xxmy = P.src(AX, AXMY);
  s.x0 = P.src(AX, AZ);
  s.s0x = P.src(AZ, AX);
  s.y0 = P.src(AY, AZ);
  s.s0y = P.src(AZ, AY);
  s.xmy0 = with_xmy0 ? P.src(AXMY, AZ) : -1;
  s.s0xmy = P.src(AZ, AXMY);
  return s;
}

/* compute_con_kernels, con_kernel.c:167-254 (struct QED_Kernels) */
void prog_con(PB &P)
{
  const ConSrc s = con_sources(P, true);
  const int l0xy = P.slot(0, 1.0, {T(s.xy), T(s.yx, NML), T(s.xxmy, LNM, -1)});
  const int l0yx = P.slot(1, 1.0, {T(s.xxmy, LNM)});
  const int b1 = P.slot(-1, 2.0, {T(s.x0, LNM), T(s.y0, LNM), T(s.x0, LMN), T(s.y0, LMN),
                                  T(s.x0, I, -1), T(s.xmy0, I, -1)});
  P.slot(2, 1.0, {T(l0xy), T(b1)});
  const int b1y = P.slot(-1, 2.0, {T(s.x0), T(s.xmy0)});
  P.slot(3, 1.0, {T(l0yx), T(b1y)});
  const int b2 = P.slot(-1, 1.0, {T(s.s0y), T(s.x0), T(s.s0x, NML), T(s.y0, NML),
                                  T(s.s0xmy, LNM, -1), T(s.x0, LNM, -1)});
  const int l2xy = P.slot(4, 1.0, {T(l0xy), T(b2, I, -1)});
  const int b2y = P.slot(-1, 1.0, {T(s.x0, LNM), T(s.s0xmy, LNM)});
  P.slot(5, 1.0, {T(l0yx), T(b2y, I, -1)});
  const int b3 = P.slot(-1, 1.0, {T(s.s0x), T(s.s0y, NML), T(s.y0, LMN), T(s.s0x, LNM, -1),
                                  T(s.y0, NML)});
  P.slot(6, 1.0, {T(l2xy), T(b3)});
  const int b3y = P.slot(-1, 1.0, {T(s.x0), T(s.s0x, LNM), T(s.s0xmy, LNM, -1)});
  P.slot(7, 1.0, {T(l0yx), T(b3y)});
}

/* compute_con_kernels_v2, con_kernel.c:61-165 (struct Kernels[3]; output
   block k * 4 + l is K[k].L<l>) */
void prog_con_v2(PB &P)
{
  const ConSrc s = con_sources(P, true);
  const int A0 = P.slot(0, 1.0, {T(s.xy)});
  const int B0 = P.slot(4, 1.0, {T(s.xxmy, LNM)});
  P.slot(8, 1.0, {T(A0), T(s.yx, NML), T(s.xxmy, LNM, -1)});
  const int a1 = P.slot(-1, 2.0, {T(s.x0, LNM), T(s.y0, LNM)});
  const int A1 = P.slot(1, 1.0, {T(A0), T(a1)});
  const int b1 = P.slot(-1, 2.0, {T(s.x0), T(s.xmy0)});
  const int B1 = P.slot(5, 1.0, {T(B0), T(b1)});
  const int c1 = P.slot(-1, 2.0, {T(s.y0, LMN), T(s.x0, LMN)});
  P.slot(9, 1.0, {T(A1), T(B1, I, -1), T(s.yx, NML), T(c1)});
  const int a2 = P.slot(-1, 1.0, {T(s.s0y), T(s.x0)});
  const int A2 = P.slot(2, 1.0, {T(A0), T(a2, I, -1)});
  const int b2 = P.slot(-1, 1.0, {T(s.s0xmy, LNM), T(s.x0, LNM)});
  const int B2 = P.slot(6, 1.0, {T(B0), T(b2, I, -1)});
  const int c2 = P.slot(-1, 1.0, {T(s.s0x, NML), T(s.y0, NML)});
  P.slot(10, 1.0, {T(A2), T(B2, I, -1), T(s.yx, NML), T(c2, I, -1)});
  const int a3 = P.slot(-1, 1.0, {T(s.x0, LNM), T(s.s0x), T(s.s0y, I, -1)});
  const int A3 = P.slot(3, 1.0, {T(A0), T(a3)});
  const int b3 = P.slot(-1, 1.0, {T(s.x0), T(s.s0x, LNM), T(s.s0xmy, LNM, -1)});
  const int B3 = P.slot(7, 1.0, {T(B0), T(b3)});
  const int c3 = P.slot(-1, 1.0, {T(s.y0, LMN), T(s.s0y, NML), T(s.s0x, NML, -1)});
  P.slot(11, 1.0, {T(A3), T(B3, I, -1), T(s.yx, NML), T(c3)});
}

/* compute_con_kernelsM_L2 (con_kernel.c:258-399, sub false) and
   compute_sub_kernelsM_L2 (sub_kernel.c:27-167, sub true) */
void prog_conM(PB &P, bool sub)
{
  const ConSrc s = con_sources(P, false);
  for (int m = 0; m < 4; m++) {
    const int lxy = P.slot(m, 1.0, {T(s.xy), G(s.s0y, I, -1, GX, m, VX, MU, VX, 0),
                                    G(s.x0, I, -1, GY, m, VY, NU, VY, 1)});
    const int lyx = P.slot(-1, 1.0, {T(s.yx, NML), G(s.s0x, NML, -1, GY, m, VY, NU, VY, 0),
                                     G(s.y0, NML, -1, GX, m, VX, MU, VX, 1)});
    const int lxxmy =
        sub ? P.slot(4 + m, 1.0, {T(s.xxmy, NLM), G(s.s0xmy, NLM, -1, GX, m, VX, NU, VX, 0),
                                  G(s.x0, NLM, -1, GXMY, m, VXMY, LA, VXMY, 1)})
            : P.slot(4 + m, 1.0, {T(s.xxmy, LNM), G(s.s0xmy, LNM, -1, GX, m, VX, LA, VX, 0),
                                  G(s.x0, LNM, -1, GXMY, m, VXMY, NU, VXMY, 1)});
    P.slot(8 + m, 1.0, {T(lxy), T(lyx), T(lxxmy, I, -1)});
  }
}

/* compute_all_kernels_SYMXY (SYMXY.c:44-85, v2 false) and _v2 (SYMXY.c:14-40) */
void prog_symxy(PB &P, bool v2)
{
  int W[8];
  prog_all_slots(P, false, W);
  int xy[4];
  for (int l = 0; l < 4; l++)
    xy[l] = P.slot(v2 ? l : 2 * l, 2.0, {T(W[2 * l]), T(W[2 * l + 1], NML)});
  if (!v2)
    for (int l = 0; l < 4; l++) P.slot(2 * l + 1, 1.0, {T(xy[l], NML)});
}

/* compute_all_kernels_SYMXY0 (SYMXY0.c:116-211, v2 false) and _v2 (SYMXY0.c:22-112) */
void prog_symxy0(PB &P, bool v2)
{
  const int sxy = P.src(AX, AY), syx = P.src(AY, AX), sxmy_x = P.src(AXMY, AX),
            symx_y = P.src(AYMX, AY), sx_xmy = P.src(AX, AXMY), sy_ymx = P.src(AY, AYMX),
            sx0 = P.src(AX, AZ), s0x = P.src(AZ, AX), sy0 = P.src(AY, AZ), s0y = P.src(AZ, AY),
            sxmy0 = P.src(AXMY, AZ), s0xmy = P.src(AZ, AXMY);
  auto o = [&](int l) { return v2 ? l : 2 * l; };
  const int l0 = P.slot(o(0), 6.0, {T(sxy), T(syx, NML), T(sxmy_x, NLM, -1), T(symx_y, MLN, -1),
                                    T(sx_xmy, LNM, -1), T(sy_ymx, LMN, -1)});
  const int apc = P.slot(-1, 1.0, {T(sx0), T(sx0, LNM, -1), T(sy0, NML), T(sy0, LMN, -1)});
  const int b1 = P.slot(-1, 12.0, {T(apc, I, -1), T(sx0, LMN), T(sx0, MLN, -1), T(sy0, LNM),
                                   T(sy0, NLM, -1), T(sxmy0, NML), T(sxmy0, I, -1), T(sxmy0, NLM),
                                   T(sxmy0, MLN, -1)});
  const int l1 = P.slot(o(1), 1.0, {T(l0), T(b1)});
  const int b2 = P.slot(-1, 6.0, {T(apc), T(s0x, NML), T(s0x, NLM, -1), T(s0y), T(s0y, MLN, -1),
                                  T(sxmy0, MLN), T(sxmy0, NLM, -1), T(s0xmy, LMN),
                                  T(s0xmy, LNM, -1)});
  const int l2 = P.slot(o(2), 1.0, {T(l0), T(b2, I, -1)});
  const int b3 = P.slot(-1, 6.0, {T(s0x), T(s0x, LNM, -1), T(s0y, NML), T(s0y, LMN, -1),
                                  T(s0xmy, MLN), T(s0xmy, NLM, -1)});
  const int l3 = P.slot(o(3), 1.0, {T(l2), T(b3)});
  if (!v2) {
    const int ls[4] = {l0, l1, l2, l3};
    for (int l = 0; l < 4; l++) P.slot(2 * l + 1, 1.0, {T(ls[l], NML)});
  }
}

/* QED_Mkernel_L2, kernels.c:181-231 (mass M[0]) */
void prog_mkernel(PB &P)
{
  const int sxy = P.src(AX, AY), s0y = P.src(AZ, AY), sx0 = P.src(AX, AZ);
  P.slot(0, 1.0, {T(sxy), G(s0y, I, -1, GX, 0, VX, MU, VX, 0), G(sx0, I, -1, GY, 0, VY, NU, VY, 1)});
}

struct Programs {
  CProgram p[KQED_COMPOSITE_COUNT];
  bool ok = true;
  Programs()
  {
    for (int w = 0; w < KQED_COMPOSITE_COUNT; w++) {
      PB P;
      int W[8];
      switch (w) {
      case KQED_ALL_KERNELS: prog_all_slots(P, true, W); break;
      case KQED_ALL_MKERNELS: prog_all_M(P, false); break;
      case KQED_ALL_MKERNELS_V2: prog_all_M(P, true); break;
      case KQED_CON_KERNELS: prog_con(P); break;
      case KQED_CON_KERNELS_V2: prog_con_v2(P); break;
      case KQED_CON_KERNELSM_L2: prog_conM(P, false); break;
      case KQED_SUB_KERNELSM_L2: prog_conM(P, true); break;
      case KQED_SYMXY: prog_symxy(P, false); break;
      case KQED_SYMXY_V2: prog_symxy(P, true); break;
      case KQED_SYMXY0: prog_symxy0(P, false); break;
      case KQED_SYMXY0_V2: prog_symxy0(P, true); break;
      case KQED_MKERNEL_L2: prog_mkernel(P); break;
      }
      if (P.bad || P.p.nout * kComp != (int)kqed_composite_size(w)) ok = false;
      p[w] = P.p;
    }
  }
};

const Programs &programs()
{
  static const Programs P;
  return P;
}

bool needs_mass(int which)
{
  return which == KQED_ALL_MKERNELS || which == KQED_ALL_MKERNELS_V2 ||
         which == KQED_CON_KERNELSM_L2 || which == KQED_SUB_KERNELSM_L2 ||
         which == KQED_MKERNEL_L2;
}

/* ------------------------------------------------------------- kernels */

__device__ __forceinline__ double arg_comp(int code, const double *x, const double *y, int k)
{
  switch (code) {
  case AX: return x[k];
  case AY: return y[k];
  case AXMY: return __dsub_rn(x[k], y[k]);
  case AYMX: return -__dsub_rn(x[k], y[k]);
  case AMY: return -y[k];
  default: return 0.0;
  }
}

/* X[j][i][4], Y[j][i][4]: the arguments of source j for pair i */
__global__ void derive_kernel(const __grid_constant__ CProgram P, const double *__restrict__ x,
                              const double *__restrict__ y, size_t n, double *__restrict__ X,
                              double *__restrict__ Y)
{
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * P.nsrc) return;
  const int j = (int)(t / n);
  const size_t i = t - (size_t)j * n;
  const double *xv = x + 4 * i, *yv = y + 4 * i;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    X[4 * t + k] = arg_comp(P.a[j], xv, yv, k);
    Y[4 * t + k] = arg_comp(P.b[j], xv, yv, k);
  }
}

__device__ __forceinline__ int lorentz(int opack, int k) { return (opack >> (2 * k)) & 3; }

/* one block per pair, one thread per component; S = the pair's sources and
   slots in shared memory, [nsrc + nslot][384], then the contraction tables
   [ncon][96].  Per pair, once: the Gaussian factors, M[mass] * u[i] and
   coef * e_g[mass] of every Gaussian term, and every contraction table, so
   that a Gaussian term costs each component one product, one difference,
   one product and the sum (the reference's order of operations). */
template <bool FUSED>
__global__ void __launch_bounds__(kComp) combine_kernel(const __grid_constant__ CProgram P,
                                                        const double *__restrict__ Tsrc, size_t n,
                                                        const double *__restrict__ x,
                                                        const double *__restrict__ y,
                                                        double *__restrict__ out)
{
  extern __shared__ double S[];
  __shared__ double vec[4][4];      /* VN, VX, VY, VXMY */
  __shared__ double gau[4][4];      /* [Gau][mass] */
  __shared__ double mu[4][4][4];    /* [mass][Vec][i] = M[mass] * vec[Vec][i] */
  __shared__ double cg[kMaxTerm];   /* coef * e_g[mass] of the Gaussian terms */
  double *CT = S + (P.nsrc + P.nslot) * kComp;
  const size_t i = blockIdx.x;
  const int c = threadIdx.x;
  for (int j = 0; j < P.nsrc; j++) S[j * kComp + c] = Tsrc[((size_t)j * n + i) * kComp + c];
  if (c < 4) {
    const double xv = x[4 * i + c], yv = y[4 * i + c];
    vec[0][c] = 0.0;
    vec[1][c] = xv;
    vec[2][c] = yv;
    vec[3][c] = __dsub_rn(xv, yv);
  }
  __syncthreads();
  if (c < 16) {
    const int g = c >> 2, m = c & 3;
    if (g == 0) {
      gau[0][m] = 1.0;
    } else {
      const double *v = vec[g];
      const double sq = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])),
                                            __dmul_rn(v[2], v[2])),
                                  __dmul_rn(v[3], v[3]));
      gau[g][m] = exp(__ddiv_rn(__dmul_rn(-P.M[m], sq), 2.0));
    }
  } else if (c >= 64 && c < 128) {
    const int k = c - 64, m = k >> 4, v = (k >> 2) & 3, e = k & 3;
    mu[m][v][e] = __dmul_rn(P.M[m], vec[v][e]);
  }
  /* contraction tables (sources only: they are complete after the first barrier) */
  for (int e = c; e < P.ncon * kConLen; e += kComp) {
    const CCon cc = P.con[e / kConLen];
    const int r = e % kConLen, rs = r >> 4, a = (r >> 2) & 3, b = r & 3;
    const int stride = cc.wpos == 0 ? 16 : (cc.wpos == 1 ? 4 : 1);
    const int base = rs * 64 + (cc.wpos == 0 ? a * 4 + b : (cc.wpos == 1 ? a * 16 + b : a * 16 + b * 4));
    const double *src = S + cc.src * kComp;
    const double *w = vec[cc.w];
    CT[e] = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(w[0], src[base]),
                                          __dmul_rn(w[1], src[base + stride])),
                                __dmul_rn(w[2], src[base + 2 * stride])),
                      __dmul_rn(w[3], src[base + 3 * stride]));
  }
  __syncthreads();
  if (c < P.nterm && P.term[c].g != G1)
    cg[c] = __dmul_rn(P.term[c].coef, gau[P.term[c].g][P.term[c].mass]);
  __syncthreads();
  const int rs = c >> 6;
  const int opack = ((c >> 4) & 3) | (((c >> 2) & 3) << 2) | ((c & 3) << 4);
  for (int s = 0; s < P.nslot; s++) {
    const CSlot sl = P.slot[s];
    double acc = 0.0;
    for (int k = 0; k < sl.count; k++) {
      const int ti = sl.first + k;
      const CTerm t = P.term[ti];
      const int i0 = lorentz(opack, t.p0), i1 = lorentz(opack, t.p1), i2 = lorentz(opack, t.p2);
      const double sv = S[t.src * kComp + rs * 64 + i0 * 16 + i1 * 4 + i2];
      double v;
      if (t.g == G1) {
        v = t.coef == 1.0 ? sv : (t.coef == -1.0 ? -sv : __dmul_rn(t.coef, sv));
      } else {
        const int ci = rs * 16 + (t.wpos == 0 ? i1 * 4 + i2 : (t.wpos == 1 ? i0 * 4 + i2 : i0 * 4 + i1));
        const double pf = CT[t.ct * kConLen + ci];
        const double m = mu[t.mass][t.u][lorentz(opack, t.uslot)];
        if (FUSED) { /* two fused multiply-adds */
          acc = fma(cg[ti], fma(-m, pf, sv), acc);
          continue;
        }
        v = __dmul_rn(cg[ti], __dsub_rn(sv, __dmul_rn(m, pf)));
      }
      acc = __dadd_rn(acc, v);
    }
    if (sl.div == 2.0) acc = __dmul_rn(acc, 0.5);   /* exact */
    else if (sl.div != 1.0) acc = __ddiv_rn(acc, sl.div);
    S[(P.nsrc + s) * kComp + c] = acc;
    if (sl.out >= 0) out[(i * P.nout + sl.out) * kComp + c] = acc;
    __syncthreads();
  }
}

size_t combine_smem(const CProgram &P)
{
  return ((size_t)(P.nsrc + P.nslot) * kComp + (size_t)P.ncon * kConLen) * sizeof(double);
}

/* pairs per launch group: the sources of one group, nsrc * chunk * (8 + 384)
   doubles, stay at about 1.2 GB or less */
constexpr size_t kChunk = (size_t)1 << 15;

int composite_dev(const struct QED_kernel_temps *t, int which, const double *M, size_t n,
                  const double *dx, const double *dy, double *dout, int precision,
                  cudaStream_t s)
{
  if (which < 0 || which >= KQED_COMPOSITE_COUNT) return set_error("unknown composite kernel");
  const Programs &PR = programs();
  if (!PR.ok) return set_error("composite kernel programs failed their self-check");
  if (precision != KQED_FP64 && precision != KQED_FP32_MIXED)
    return set_error("composite kernels: precision must be KQED_FP64 or KQED_FP32_MIXED");
  CProgram P = PR.p[which];
  if (needs_mass(which)) {
    if (!M) return set_error("this composite kernel needs its masses M");
    const int nm = which == KQED_MKERNEL_L2 ? 1 : 4;
    for (int k = 0; k < nm; k++) P.M[k] = M[k];
  }
  if (n == 0) return 0;
  if (!dx || !dy || !dout) return set_error("null buffer");
  const size_t chunk = std::min(n, kChunk);
  const size_t per = (size_t)P.nsrc * chunk;
  double *scr = stage_scratch(t, 0, per * (8 + kComp));
  if (!scr) return set_error("out of device memory for the composite kernels' sources");
  double *X = scr, *Y = scr + 4 * per, *Tsrc = scr + 8 * per;
  const size_t smem = combine_smem(P);
  /* the attribute is per function: set the largest any program needs, so
     that concurrent callers with different programs never lower it */
  const void *cfn = precision == KQED_FP64 ? (const void *)combine_kernel<false>
                                           : (const void *)combine_kernel<true>;
  if (cudaFuncSetAttribute(cfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(((kMaxSrc + kMaxSlot) * kComp + kMaxCon * kConLen) *
                                 sizeof(double))) != cudaSuccess)
    return set_error("composite kernels: shared memory attribute refused");
  const size_t osz = (size_t)P.nout * kComp;
  for (size_t p0 = 0; p0 < n; p0 += chunk) {
    const size_t m = std::min(chunk, n - p0);
    const size_t th = m * P.nsrc;
    derive_kernel<<<(unsigned)((th + 255) / 256), 256, 0, s>>>(P, dx + 4 * p0, dy + 4 * p0, m, X, Y);
    if (cudaGetLastError() != cudaSuccess) return set_error("composite derive launch failed");
    g_launches++;
    if (l0_pairs(t, X, Y, th, Tsrc, precision, s)) return 1;
    if (precision == KQED_FP64)
      combine_kernel<false><<<(unsigned)m, kComp, smem, s>>>(P, Tsrc, m, dx + 4 * p0, dy + 4 * p0,
                                                             dout + p0 * osz);
    else
      combine_kernel<true><<<(unsigned)m, kComp, smem, s>>>(P, Tsrc, m, dx + 4 * p0, dy + 4 * p0,
                                                            dout + p0 * osz);
    if (cudaGetLastError() != cudaSuccess) return set_error("composite combine launch failed");
    g_launches++;
  }
  return 0;
}

/* host buffers, in groups of kChunk pairs */
int composite_host(const struct QED_kernel_temps *t, int which, const double *M, size_t n,
                   const double *x, const double *y, double *out, int precision)
{
  if (which < 0 || which >= KQED_COMPOSITE_COUNT) return set_error("unknown composite kernel");
  if (n == 0) return 0;
  if (!x || !y || !out) return set_error("null buffer");
  cudaStream_t s = stage_stream(t);
  if (!s) return set_error("tables not initialised");
  const size_t osz = kqed_composite_size(which);
  if (n > SIZE_MAX / (sizeof(double) * (osz + 8))) return set_error("too many pairs");
  /* an output in kqed_pinned_alloc memory is written in place by the
     combine kernel; then one pass over all pairs, one synchronisation */
  if (double *oin = static_cast<double *>(pinned_device(out, n * osz * sizeof(double)))) {
    double *io = stage_scratch(t, 1, 8 * n);
    if (!io) return set_error("out of device memory for composite kernel staging");
    if (cudaMemcpyAsync(io, x, n * 4 * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(io + 4 * n, y, n * 4 * sizeof(double), cudaMemcpyHostToDevice, s) !=
            cudaSuccess)
      return set_error("composite kernels: copy to the device failed");
    if (composite_dev(t, which, M, n, io, io + 4 * n, oin, precision, s)) return 1;
    if (cudaStreamSynchronize(s) != cudaSuccess) return set_error("composite kernels: execution failed");
    return 0;
  }
  const size_t chunk = std::min(n, kChunk);
  double *io = stage_scratch(t, 1, chunk * (8 + osz));
  if (!io) return set_error("out of device memory for composite kernel staging");
  double *dx = io, *dy = io + 4 * chunk, *dk = io + 8 * chunk;
  for (size_t p0 = 0; p0 < n; p0 += chunk) {
    const size_t m = std::min(chunk, n - p0);
    if (cudaMemcpyAsync(dx, x + 4 * p0, m * 4 * sizeof(double), cudaMemcpyHostToDevice, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(dy, y + 4 * p0, m * 4 * sizeof(double), cudaMemcpyHostToDevice, s) !=
            cudaSuccess)
      return set_error("composite kernels: copy to the device failed");
    if (composite_dev(t, which, M, m, dx, dy, dk, precision, s)) return 1;
    if (cudaMemcpyAsync(out + p0 * osz, dk, m * osz * sizeof(double), cudaMemcpyDeviceToHost,
                        s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return set_error("composite kernels: copy back or execution failed");
  }
  return 0;
}

/* the reference-signature calls: one pair, errors on stderr and a zero
   output, like the per-pair kernel calls */
void composite_one(const char *name, int which, const double *M, const double xv[4],
                   const double yv[4], const struct QED_kernel_temps &t, void *out)
{
  const size_t sz = kqed_composite_size(which);
  if (composite_host(&t, which, M, 1, xv, yv, static_cast<double *>(out), KQED_FP64)) {
    fprintf(stderr, "%s: %s\n", name, kqed_last_error());
    memset(out, 0, sz * sizeof(double));
  }
}

} // namespace
} // namespace kqed

using kqed::composite_one;

/* ------------------------------------------------------------- C ABI */

extern "C" size_t kqed_composite_size(int which)
{
  switch (which) {
  case KQED_ALL_KERNELS: case KQED_ALL_MKERNELS: case KQED_ALL_MKERNELS_V2:
  case KQED_CON_KERNELS: case KQED_SYMXY: case KQED_SYMXY0:
    return sizeof(struct QED_Kernels) / sizeof(double);
  case KQED_CON_KERNELS_V2: case KQED_CON_KERNELSM_L2: case KQED_SUB_KERNELSM_L2:
    return 3 * sizeof(struct Kernels) / sizeof(double);
  case KQED_SYMXY_V2: case KQED_SYMXY0_V2:
    return sizeof(struct Kernels) / sizeof(double);
  case KQED_MKERNEL_L2:
    return 384;
  default:
    return 0;
  }
}

extern "C" int kqed_composite_batch_dev(const struct QED_kernel_temps *t, int which,
                                        const double *M, size_t n, const double *d_x,
                                        const double *d_y, double *d_out, int precision,
                                        void *stream)
{
  if (!t || !t->Grid.PC) return kqed::set_error("tables not initialised");
  return kqed::composite_dev(t, which, M, n, d_x, d_y, d_out, precision, (cudaStream_t)stream);
}

extern "C" int kqed_composite_batch(const struct QED_kernel_temps *t, int which, const double *M,
                                    size_t n, const double *x, const double *y, double *out,
                                    int precision)
{
  if (!t || !t->Grid.PC) return kqed::set_error("tables not initialised");
  return kqed::composite_host(t, which, M, n, x, y, out, precision);
}

extern "C" void compute_all_kernels(const double xv[4], const double yv[4],
                                    const struct QED_kernel_temps t, struct QED_Kernels *K)
{
  composite_one("compute_all_kernels", KQED_ALL_KERNELS, nullptr, xv, yv, t, K);
}
extern "C" void compute_all_Mkernels(const double M[4], const double xv[4], const double yv[4],
                                     const struct QED_kernel_temps t, struct QED_Kernels *K)
{
  composite_one("compute_all_Mkernels", KQED_ALL_MKERNELS, M, xv, yv, t, K);
}
extern "C" void compute_all_Mkernels_v2(const double M[4], const double xv[4], const double yv[4],
                                        const struct QED_kernel_temps t, struct QED_Kernels *K)
{
  composite_one("compute_all_Mkernels_v2", KQED_ALL_MKERNELS_V2, M, xv, yv, t, K);
}
extern "C" void compute_con_kernels(const double xv[4], const double yv[4],
                                    const struct QED_kernel_temps t, struct QED_Kernels *K)
{
  composite_one("compute_con_kernels", KQED_CON_KERNELS, nullptr, xv, yv, t, K);
}
extern "C" void compute_con_kernels_v2(const double xv[4], const double yv[4],
                                       const struct QED_kernel_temps t, struct Kernels *K)
{
  composite_one("compute_con_kernels_v2", KQED_CON_KERNELS_V2, nullptr, xv, yv, t, K);
}
extern "C" void compute_con_kernelsM_L2(const double M[4], const double xv[4], const double yv[4],
                                        const struct QED_kernel_temps t, struct Kernels *K)
{
  composite_one("compute_con_kernelsM_L2", KQED_CON_KERNELSM_L2, M, xv, yv, t, K);
}
extern "C" void compute_sub_kernelsM_L2(const double M[4], const double xv[4], const double yv[4],
                                        const struct QED_kernel_temps t, struct Kernels *K)
{
  composite_one("compute_sub_kernelsM_L2", KQED_SUB_KERNELSM_L2, M, xv, yv, t, K);
}
extern "C" void compute_all_kernels_SYMXY(const double xv[4], const double yv[4],
                                          const struct QED_kernel_temps t, struct QED_Kernels *K)
{
  composite_one("compute_all_kernels_SYMXY", KQED_SYMXY, nullptr, xv, yv, t, K);
}
extern "C" void compute_all_kernels_SYMXY_v2(const double xv[4], const double yv[4],
                                             const struct QED_kernel_temps t, struct Kernels *K)
{
  composite_one("compute_all_kernels_SYMXY_v2", KQED_SYMXY_V2, nullptr, xv, yv, t, K);
}
extern "C" void compute_all_kernels_SYMXY0(const double xv[4], const double yv[4],
                                           const struct QED_kernel_temps t, struct QED_Kernels *K)
{
  composite_one("compute_all_kernels_SYMXY0", KQED_SYMXY0, nullptr, xv, yv, t, K);
}
extern "C" void compute_all_kernels_SYMXY0_v2(const double xv[4], const double yv[4],
                                              const struct QED_kernel_temps t, struct Kernels *K)
{
  composite_one("compute_all_kernels_SYMXY0_v2", KQED_SYMXY0_V2, nullptr, xv, yv, t, K);
}
extern "C" void QED_Mkernel_L2(const double M, const double xv[4], const double yv[4],
                               const struct QED_kernel_temps t, double kerv[6][4][4][4])
{
  composite_one("QED_Mkernel_L2", KQED_MKERNEL_L2, &M, xv, yv, t, kerv);
}

/* average_all_kernels, all_kernels.c:19-43: K = (K + W) / 2 */
extern "C" void average_all_kernels(struct Kernels *K, const struct Kernels W)
{
  double *k = &K->L0[0][0][0][0];
  const double *w = &W.L0[0][0][0][0];
  for (int i = 0; i < 4 * 384; i++) k[i] = 0.5 * (k[i] + w[i]);
}

/* average_all_QED_kernels, all_kernels.c:46-82 */
extern "C" void average_all_QED_kernels(struct QED_Kernels *K, const struct QED_Kernels W)
{
  double *k = &K->L0.xy[0][0][0][0];
  const double *w = &W.L0.xy[0][0][0][0];
  for (int i = 0; i < 8 * 384; i++) k[i] = 0.5 * (k[i] + w[i]);
}

/* average_con_kernels, con_kernel.c:14-59: K[0..2] = (K[0..2] + W[0..2]) / 2 */
extern "C" void average_con_kernels(struct Kernels *K, const struct Kernels *W)
{
  double *k = &K[0].L0[0][0][0][0];
  const double *w = &W[0].L0[0][0][0][0];
  for (int i = 0; i < 3 * 4 * 384; i++) k[i] = 0.5 * (k[i] + w[i]);
}

/* swap_munu_Lyx, all_kernels.c:373-406: every L<i>.yx gets mu <-> nu */
extern "C" void swap_munu_Lyx(struct QED_Kernels *K)
{
  struct Kernel *ks[4] = {&K->L0, &K->L1, &K->L2, &K->L3};
  for (int l = 0; l < 4; l++)
    for (int rs = 0; rs < 6; rs++)
      for (int mu = 0; mu < 4; mu++)
        for (int nu = mu + 1; nu < 4; nu++)
          for (int la = 0; la < 4; la++) {
            const double t = ks[l]->yx[rs][nu][mu][la];
            ks[l]->yx[rs][nu][mu][la] = ks[l]->yx[rs][mu][nu][la];
            ks[l]->yx[rs][mu][nu][la] = t;
          }
}
