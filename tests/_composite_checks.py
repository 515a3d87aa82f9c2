"""The reference's own identity tests of its composite kernels
(src/amu_forlattice.c, examples 12-21 and 23), restated over an evaluator so
that the same checks run on the oracle (CPU) and on the GPU library.

comp(which, x, y, M) -> [n][size] in the reference's struct layout;
kern(variant, x, y) -> [n][384] for QED_kernel_L<variant>.  The reference
compares with an absolute 1e-12 on kernels of order one; here every check is
|a - b| <= TOL * scale per pair, scale = the largest |L0| the compared
composites combine (composite_scale)."""
import numpy as np

from _helpers import composite_scale

TOL = 1e-12
(ALL, ALLM, ALLM2, CON, CON2, CONM, SUBM, SYMXY, SYMXY2, SYMXY0, SYMXY02, MKER) = range(12)


def qk(a):
    """struct QED_Kernels -> [n][L][xy|yx][6][4][4][4]"""
    return a.reshape(-1, 4, 2, 6, 4, 4, 4)


def ks(a):
    """struct Kernels (or Kernels[3]) -> [n][(k)][L][6][4][4][4]"""
    return a.reshape(-1, 4, 6, 4, 4, 4) if a.shape[1] == 1536 else a.reshape(-1, 3, 4, 6, 4, 4, 4)


def perm(a, src):
    """B[..., j, k, l] = A[..., <src>], src a permutation of 'jkl'"""
    return np.einsum("..." + src + "->...jkl", a)


def close(a, b, scale, what):
    n = len(scale)
    d = np.abs(np.asarray(a) - np.asarray(b)).reshape(n, -1).max(1)
    bad = d > TOL * scale
    assert not bad.any(), (what, float((d / scale).max()), np.nonzero(bad)[0])


def check_all(comp, kern, x, y, scale):
    """example 12 (src/amu_forlattice.c:475-540): compute_all_kernels gives
    L<v>(x,y) and L<v>(y,x)"""
    K = qk(comp(ALL, x, y, None))
    for v in range(4):
        close(K[:, v, 0], kern(v, x, y).reshape(-1, 6, 4, 4, 4), scale, "L%d.xy" % v)
        close(K[:, v, 1], kern(v, y, x).reshape(-1, 6, 4, 4, 4), scale, "L%d.yx" % v)


def check_symxy(comp, x, y, scale):
    """example 13 (:542-595): SYMXY(x,y)_{mu nu} = SYMXY(y,x)_{nu mu}"""
    a, b = ks(comp(SYMXY2, x, y, None)), ks(comp(SYMXY2, y, x, None))
    close(a, perm(b, "kjl"), scale, "SYMXY")


def check_symxy0(comp, x, y, scale):
    """example 14 (:597-742): the full symmetry of SYMXY0 under the six
    argument orders, and example 16 (:744-818): SYMXY0 as the average of
    compute_all_kernels at (x,y), (x,x-y), (y,y-x)"""
    xmy, ymx = x - y, -(x - y)
    S = lambda a, b: ks(comp(SYMXY02, a, b, None))
    k1xy = S(x, y)
    close(k1xy, perm(S(y, x), "kjl"), scale, "SYMXY0 (y,x)")
    close(k1xy, -perm(S(x, xmy), "lkj"), scale, "SYMXY0 (x,x-y)")
    close(k1xy, -perm(S(xmy, x), "klj"), scale, "SYMXY0 (x-y,x)")
    close(k1xy, -perm(S(y, ymx), "ljk"), scale, "SYMXY0 (y,y-x)")
    close(k1xy, -perm(S(ymx, y), "jlk"), scale, "SYMXY0 (y-x,y)")
    A = lambda a, b: qk(comp(ALL, a, b, None))
    K1, K2, K3 = A(x, y), A(x, xmy), A(y, ymx)
    avg = (K1[:, :, 0] + perm(K1[:, :, 1], "kjl") - perm(K2[:, :, 0], "lkj") -
           perm(K2[:, :, 1], "klj") - perm(K3[:, :, 0], "ljk") - perm(K3[:, :, 1], "jlk")) / 6.
    close(k1xy, avg, scale, "SYMXY0 average")


def check_con(comp, x, y, scale):
    """example 17 (:820-911) and 18 (:913-1013): compute_con_kernels and _v2
    from compute_all_kernels at (x,y) and (x,x-y)"""
    K1 = qk(comp(CON, x, y, None))
    K2, K3 = qk(comp(ALL, x, y, None)), qk(comp(ALL, x, x - y, None))
    C = K2[:, :, 0] + perm(K2[:, :, 1], "kjl") - perm(K3[:, :, 0], "lkj")
    close(K1[:, :, 0], C, scale, "con xy")
    close(K1[:, :, 1], perm(K3[:, :, 0], "lkj"), scale, "con yx")
    V = ks(comp(CON2, x, y, None))
    close(V[:, 0], K2[:, :, 0], scale, "con_v2 A")
    close(V[:, 1], perm(K3[:, :, 0], "lkj"), scale, "con_v2 B")
    close(V[:, 2], C, scale, "con_v2 C")


def check_mkernels(comp, kern, x, y, scale):
    """example 20 (:1080-1158): compute_con_kernelsM_L2 from QED_Mkernel_L2
    (and the same for compute_sub_kernelsM_L2 with its own index order);
    example 21 (:1160-1228): compute_all_Mkernels at M = 0 is L2, at M[1]
    QED_Mkernel_L2; example 23 (:1246-1300): the _v2 combinations"""
    M = np.array([0.0, 0.5, 1.0, 1.5])
    xmy = x - y
    Mk = lambda m, a, b: comp(MKER, a, b, np.array([m])).reshape(-1, 6, 4, 4, 4)
    for which, order in ((CONM, "lkj"), (SUBM, "klj")):
        K = ks(comp(which, x, y, M))
        for m in range(4):
            k1, k2, k3 = Mk(M[m], x, y), Mk(M[m], y, x), Mk(M[m], x, xmy)
            close(K[:, 0, m], k1, scale, "M-kernel %d A" % which)
            close(K[:, 1, m], perm(k3, order), scale, "M-kernel %d B" % which)
            close(K[:, 2, m], k1 + perm(k2, "kjl") - perm(k3, order), scale, "M-kernel %d C" % which)
    M = np.array([0.0, 0.4, 0.8, 1.2])
    A = qk(comp(ALLM, x, y, M))
    close(A[:, 0, 0], kern(2, x, y).reshape(-1, 6, 4, 4, 4), scale, "all_Mkernels M=0 xy")
    close(A[:, 0, 1], kern(2, y, x).reshape(-1, 6, 4, 4, 4), scale, "all_Mkernels M=0 yx")
    close(A[:, 1, 0], Mk(M[1], x, y), scale, "all_Mkernels M1 xy")
    close(A[:, 1, 1], Mk(M[1], y, x), scale, "all_Mkernels M1 yx")
    B = qk(comp(ALLM2, x, y, M))
    close(B[:, 1, 0], A[:, 1, 0] + perm(A[:, 1, 1], "kjl"), scale, "all_Mkernels_v2 xy")
    close(B[:, 1, 1], Mk(M[1], x, -y), scale, "all_Mkernels_v2 yx")


def identity_scale(x, y, l0):
    """scale covering every L0 the identities combine (all derived
    arguments of the pairs and of the re-ordered calls)"""
    s = np.zeros(len(x))
    for a, b in ((x, y), (x, x - y), (y, -(x - y)), (x, -y)):
        for w in (ALLM2, CON, SYMXY0):
            s = np.maximum(s, composite_scale(w, a, b, l0))
            s = np.maximum(s, composite_scale(w, b, a, l0))
    return s


def run_all(comp, kern, x, y, l0):
    scale = identity_scale(x, y, l0)
    check_all(comp, kern, x, y, scale)
    check_symxy(comp, x, y, scale)
    check_symxy0(comp, x, y, scale)
    check_con(comp, x, y, scale)
    check_mkernels(comp, kern, x, y, scale)
