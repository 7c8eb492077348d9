"""GroupwiseRegistration restated in numpy, float32 -- TEST INFRASTRUCTURE
(oracle).  Parity pinned: tests/test_registration.py compares it with the
reference's own kernels run on the host (oracle/refkernels/
registration_host.hpp, fixtures in tests/golden/registration_*.npz).

This is the algorithm the reference's ~35 kernels compute, written per
quantity instead of per kernel, with the reference's index quirks kept where
they change the result (each noted where it is restated):

  x_d(p)        identity mesh, 1-based (col + 1, row + 1)
  u_d,f(p)      = sum_{a,b} T[d][f][cr(row)+b][cc(col)+a] B(row,b) B(col,a)   (FFD)
  xn            = x + u inside the bounding box, x outside
  I_w           = bilinear(I, xn) on the margin rectangle, I elsewhere
  V(p)          = var_f I_w(p)  [+ smoothness terms when sumLambda() != 0]
  H             = sum_{p in ROI} V(p)
  dH[d][f][k][l]= sum_{support of (k, l)} ROI (dy dx_d S(i) S(j) + aux2[k][l][i][j])
  T            -= Wn (dH - mean_f dH)

Symbols follow GroupwiseRegistration.cpp / optimizer.cl.  Square images and a
circular region of interest only (the reference's grid and mask assume a
square image; its whole-box mode stores a degenerate bounding box).
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


# ---- groupwiseRegistration/bspline.cpp (float results of double arithmetic) ----
def _bspline(t: int, x: float, E: int) -> float:
    """bsplineN / b1splineN / b2splineN (t = 0, 1, 2) of order E = 1, 2, 3,
    rounded as the reference's float and double expressions round."""
    x = float(np.float32(x))
    fx = f32(x)
    if E == 1:
        if t == 0:
            if -1 <= x < 0:
                return float(f32(fx + f32(1)))
            if 0 <= x < 1:
                return float(f32(f32(1) - fx))
            return 0.0
        if t == 1:
            return 1.0 if -1 <= x < 0 else (-1.0 if 0 <= x < 1 else 0.0)
        return 0.0
    if E == 2:
        if t == 0:
            if -1.5 <= x < -0.5:
                return float(f32((4 * math.pow(x, 2) + float(f32(12 * fx)) + 9) / 8))
            if -0.5 <= x < 0.5:
                return float(f32((-4 * math.pow(x, 2) + 3) / 4))
            if 0.5 <= x < 1.5:
                return float(f32((4 * math.pow(x, 2) - float(f32(12 * fx)) + 9) / 8))
            return 0.0
        if t == 1:
            if -1.5 <= x < -0.5:
                return float(f32(f32(f32(2 * fx) + f32(3)) / f32(2)))
            if -0.5 <= x < 0.5:
                return float(f32(-2 * fx))
            if 0.5 <= x < 1.5:
                return float(f32(f32(f32(42 * fx) - f32(3)) / f32(2)))  # the reference's constant
            return 0.0
        if -1.5 <= x < -0.5:
            return 1.0
        if -0.5 <= x < 0.5:
            return -2.0
        if 0.5 <= x < 1.5:
            return 1.0
        return 0.0
    if E == 3:
        if t == 0:
            v = abs(x)
            if v < 1:
                return float(f32(0.5 * math.pow(f32(v), 3) - math.pow(f32(v), 2) + 0.6666))
            if 1 <= v < 2:
                return float(f32(f32(f32(2 - v) * f32(2 - v)) * f32(2 - v)) / f32(6))
            return 0.0
        if t == 1:
            if 0 <= x <= 1:
                return float(f32(1.5 * math.pow(x, 2) - 2 * x))
            if -1 <= x < 0:
                return float(f32(-1.5 * math.pow(x, 2) - 2 * x))
            if 1 < x < 2:
                return float(f32(-f32(f32(x - 2) * f32(x - 2)) / f32(2)))
            if -2 < x < -1:
                return float(f32(f32(f32(x + 2) * f32(x + 2)) / f32(2)))
            return 0.0
        v = abs(x)
        if v < 1:
            return float(f32(f32(3 * f32(v)) - f32(2)))
        if 1 <= v < 2:
            return float(f32(-f32(v) + f32(2)))
        return 0.0
    raise NotImplementedError("spline orders 1 to 3")


def _round_half_away(v: float) -> float:
    """std::round: halves away from zero."""
    return float(math.floor(v + 0.5)) if v >= 0 else float(math.ceil(v - 0.5))


class Geometry:
    """init() and creabspline() (GroupwiseRegistration.cpp:92-400,
    groupwiseRegistration/creabspline.cpp) reduced to what the iteration uses."""

    def __init__(self, N: int, F: int, radius: int, E: int = 3, Dp: int = 4):
        if radius <= 0:
            raise ValueError("circular region of interest only")
        self.N, self.F, self.E, self.Dp = N, F, E, Dp
        # setMask (GroupwiseRegistration.cpp:486-531)
        center = f32((N + 1) / 2)
        j = np.arange(N)
        Cv = ((f32(1) - center + j.astype(f32)) ** 2).astype(f32)
        roi = (Cv[None, :] + Cv[:, None]) <= radius * radius  # [row][col]
        rows, cols = np.nonzero(roi)
        self.roi = roi.astype(f32)
        self.areaX = int(roi.sum())
        bb = [int(cols.min()) + 1, int(rows.min()) + 1, int(cols.max()) + 1, int(rows.max()) + 1]
        if bb[0] != bb[1] or bb[2] != bb[3]:
            raise ValueError("the region of interest must be symmetric")
        self.bb = bb
        m = N // 40
        # margin rectangle of the interpolators (Interpolator::init), 0-based
        self.rect_rows = np.arange(bb[1] - m - 2, bb[3] + m + 1)
        self.rect_cols = np.arange(bb[0] - m - 2, bb[2] + m + 1)
        c = f32((bb[0] + bb[2]) / 2)
        rp = (E + 1) * Dp // 2
        C0 = int(math.floor(f32(f32(abs(c - f32(bb[0])) + f32(rp)) / f32(Dp))))
        C1 = int(math.floor(f32(f32(abs(c - f32(bb[2])) + f32(rp)) / f32(Dp))))
        self.Cp = C0 + C1 + 1
        self.dp = 2 * int(math.ceil(rp)) + 1
        # per-pixel control ranges and spline values (coef, BBAux)
        p1 = (np.arange(N) + 1).astype(f32)
        # creabspline.cpp: odd orders floor((x - c) / Dp) - (E - 1) / 2, even orders
        # round((x - c) / Dp) - E / 2
        if E % 2:
            kmin = np.array([math.floor(f32(f32(v - c) / f32(Dp))) - (E - 1) // 2 for v in p1], np.float64)
        else:
            kmin = np.array([_round_half_away(float(f32(f32(v - c) / f32(Dp)))) - E // 2 for v in p1], np.float64)
        self.kmin = kmin
        ref = kmin[bb[0]]  # coef at index bound_box[d] (creabspline.cpp)
        self.cr = (kmin + 1 - ref - 1).astype(np.int64)  # 0-based first control point of each pixel
        self.B = np.zeros((3, N, E + 1), f32)  # [t][pixel][spline]
        for p in range(N):
            for s in range(E + 1):
                k = int(kmin[p]) + s
                arg = f32(f32(f32(f32(p + 1) - c) / f32(Dp)) - f32(k))
                for t in range(3):
                    self.B[t, p, s] = _bspline(t, arg, E)
        # control points and their supports (ControlPointsLocation, coefg, BBAux1)
        pu = (c + f32(Dp) * (np.arange(self.Cp) - C0).astype(f32)).astype(f32)
        self.pu = pu
        start = np.array([math.ceil(f32(v - f32(math.ceil(rp)))) for v in pu], np.int64)  # 1-based
        self.sup = start - 1  # 0-based first pixel of each support
        if self.sup.min() < 0 or self.sup.max() + self.dp > N:
            raise ValueError("control supports leave the image")
        S = np.zeros((3, self.Cp, self.dp), f32)
        for n in range(self.Cp):
            for s in range(self.dp):
                arg = f32(f32(f32(start[n] + s) - pu[n]) / f32(Dp))
                for t in range(3):
                    S[t, n, s] = _bspline(t, arg, E)
        if not np.all(S == S[:, :1, :]):
            raise ValueError("support splines differ between control points")
        self.S = S[:, 0, :]  # [t][offset]
        # in-box pixel ranges (rows r2, columns r1 of the reference)
        self.box_rows = np.arange(bb[1] - 1, bb[3])
        self.box_cols = np.arange(bb[0] - 1, bb[2])


def _bilinear(img: np.ndarray, xn0: np.ndarray, xn1: np.ndarray) -> np.ndarray:
    """optimizer.cl interpolator / gradientInterpolator arithmetic at 1-based
    mesh coordinates (xn0 horizontal, xn1 vertical); img [N][N]."""
    N = img.shape[-1]
    nh = (xn0 - f32(1)).astype(f32)
    nv = (xn1 - f32(1)).astype(f32)
    ph = np.floor(nh).astype(np.int64)
    pv = np.floor(nv).astype(np.int64)
    flat = img.reshape(-1)
    i1 = flat[ph + pv * N]
    i2 = flat[ph + 1 + pv * N]
    i3 = flat[ph + (pv + 1) * N]
    i4 = flat[ph + 1 + (pv + 1) * N]
    a = ((ph + 1).astype(f32) - nh).astype(f32)
    b = (nh - ph.astype(f32)).astype(f32)
    c = ((pv + 1).astype(f32) - nv).astype(f32)
    d = (nv - pv.astype(f32)).astype(f32)
    aux1 = (a * i1 + b * i2).astype(f32)
    aux2 = (a * i3 + b * i4).astype(f32)
    return (c * aux1 + d * aux2).astype(f32)


def _seqsum(terms):
    acc = None
    for t in terms:
        acc = t.astype(f32) if acc is None else (acc + t).astype(f32)
    return acc


class Registration:
    """GroupwiseRegistration::launch with optimizer() (optimizer.cpp), float32.
    images [F][N][N] complex; returns T [2][F][Cp][Cp] ([d][frame][row control
    point][column control point]), xn [2][F][N][N], H per iteration, Wn."""

    def __init__(self, N, F, radius=40, E=3, Dp=(4, 4), nmax=100, et=0.01, eh=0.005,
                 lambda_=(0.0, 0.005, 0.0, 0.5), W=1.0, flagW=True):
        if Dp[0] != Dp[1]:
            raise ValueError("equal control spacing in both directions only")
        if F < 3 or N % 8:
            raise ValueError("F >= 3 and N a multiple of 8")
        self.g = Geometry(N, F, radius, E, Dp[0])
        self.N, self.F = N, F
        self.nmax, self.et, self.eh = nmax, f32(et), f32(eh)
        self.lam = [f32(v) for v in lambda_]
        # sumLambda() adds the weights into an int (GroupwiseRegistration.cpp:440-442)
        acc = 0
        for v in lambda_:
            acc = int(acc + float(f32(v)))
        self.sum_lambda = acc
        self.Wn = f32(f32(W) / f32(self.g.areaX))
        self.flagW = flagW

    # ---- deformation (TransformationAux, Deformation, DeformationAdjust) ----
    def deform(self, T):
        g, N, F = self.g, self.N, self.F
        rows, cols = g.box_rows, g.box_cols
        B0 = g.B[0]
        xn = np.zeros((2, F, N, N), f32)
        rr, cc = np.meshgrid(rows, cols, indexing="ij")
        cr, ccp = g.cr[rr], g.cr[cc]
        for d in range(2):
            for f in range(F):
                acc = np.zeros(rr.shape, f32)
                for a in range(g.E + 1):          # Deformation kernel: m (column spline) outer
                    for b in range(g.E + 1):      # n (row spline) inner
                        bb = (B0[rr, b] * B0[cc, a]).astype(f32)
                        acc = (acc + (T[d, f][cr + b, ccp + a] * bb).astype(f32)).astype(f32)
                xn[d, f][rr, cc] = acc
        colg, rowg = np.meshgrid(np.arange(N), np.arange(N))
        xn[0] = (xn[0] + (colg + 1).astype(f32)).astype(f32)
        xn[1] = (xn[1] + (rowg + 1).astype(f32)).astype(f32)
        return xn

    def warp(self, img, xn):
        """Interpolator over the margin rectangle (CopyDataGPU elsewhere)."""
        g = self.g
        out = img.copy()
        rr, cc = np.meshgrid(g.rect_rows, g.rect_cols, indexing="ij")
        for f in range(self.F):
            out[f][rr, cc] = _bilinear(img[f], xn[0, f][rr, cc], xn[1, f][rr, cc])
        return out

    def metric(self, Iw):
        """metric kernel: mean over frames, then the variance accumulated frame by frame."""
        F = self.F
        mean = (_seqsum([Iw[f] for f in range(F)]) / f32(F)).astype(f32)
        V = np.zeros(Iw.shape[1:], f32)
        for f in range(F):
            dlt = (Iw[f] - mean).astype(f32)
            V = (V + (dlt * dlt).astype(f32)).astype(f32)
        return (V / f32(F)).astype(f32), mean

    def cost(self, V):
        """costReduction: one sequential masked sum over the pixels."""
        x = (V * self.g.roi).astype(f32).reshape(-1)
        return f32(np.cumsum(x, dtype=f32)[-1])

    # ---- regularization (PermuteTAux, ShiftTAux, Regularization) ----
    def smoothness(self, T):
        """dtau arrays as the reference stores them: value at (pixel row r,
        column c) kept at image position [r][c] of a transposed store, i.e.
        returned arrays are indexed [..][r][c] with the reference's pairing of
        spline factors (the row-direction control offset n is weighted by the
        column pixel's spline and vice versa, optimizer.cl:746-830)."""
        g, F = self.g, self.F
        N = self.N
        Dp = g.Dp
        B, B1, B2 = g.B[0], g.B[1], g.B[2]
        rows, cols = g.box_rows, g.box_cols
        rr, cc = np.meshgrid(rows, cols, indexing="ij")
        cr, ccp = g.cr[rr], g.cr[cc]
        shp = (F, N, N)
        dtaux = np.zeros((2, 2) + shp, f32)
        dtaux2 = np.zeros((2, 2) + shp, f32)
        dtauxy = np.zeros((2,) + shp, f32)
        dtaut = np.zeros((2,) + shp, f32)
        dtaut2 = np.zeros((2,) + shp, f32)
        # every (d, frame) at once; per element the same loop order and roundings
        T1a, T2a = np.roll(T, 1, axis=1), np.roll(T, 2, axis=1)      # frames f-1, f-2
        box = (2, F) + rr.shape
        ax = np.zeros((2,) + box, f32)
        ax2 = np.zeros((2,) + box, f32)
        axy = np.zeros(box, f32)
        at = np.zeros(box, f32)
        at2 = np.zeros(box, np.float64)
        E1 = g.E + 1
        for m in range(E1):
            for n in range(E1):
                t0 = T[:, :, cr + n, ccp + m]
                bx = [(f32(Dp) * (B[cc, n] * B1[rr, m]).astype(f32)).astype(f32),
                      (f32(Dp) * (B1[cc, n] * B[rr, m]).astype(f32)).astype(f32)]
                bx2 = [(f32(Dp * Dp) * (B[cc, n] * B2[rr, m]).astype(f32)).astype(f32),
                       (f32(Dp * Dp) * (B2[cc, n] * B[rr, m]).astype(f32)).astype(f32)]
                for p in range(2):
                    ax[p] = (ax[p] + (t0 * bx[p]).astype(f32)).astype(f32)
                    ax2[p] = (ax2[p] + (t0 * bx2[p]).astype(f32)).astype(f32)
        for p in range(2):  # + 1 where the derivative direction is the displacement's (p == d)
            ax[p, p] = (ax[p, p] + f32(1)).astype(f32)
        for m in range(E1):
            for n in range(E1):
                t0 = T[:, :, cr + n, ccp + m]
                bxy = (f32(Dp * Dp) * (B1[cc, n] * B1[rr, m]).astype(f32)).astype(f32)
                axy = (axy + (t0 * bxy).astype(f32)).astype(f32)
        for m in range(E1):
            for n in range(E1):
                t0, t1, t2 = T[:, :, cr + n, ccp + m], T1a[:, :, cr + n, ccp + m], T2a[:, :, cr + n, ccp + m]
                bb = (B[cc, n] * B[rr, m]).astype(f32)
                at = (at + ((t0 - t1).astype(f32) * bb).astype(f32)).astype(f32)
                at2 = (at2.astype(f32).astype(np.float64)
                       + (t0.astype(np.float64) - 2.0 * t1.astype(np.float64) + t2.astype(np.float64))
                       * bb.astype(np.float64)).astype(f32).astype(np.float64)
        dtaux[..., rr, cc] = ax
        dtaux2[..., rr, cc] = ax2
        dtauxy[..., rr, cc] = axy
        dtaut[..., rr, cc] = at
        dtaut2[..., rr, cc] = at2.astype(f32)
        return dtaux, dtaux2, dtauxy, dtaut, dtaut2

    # ---- gradient of the metric (Gradient, Initdx, GradientInterpolator, GradientMetric) ----
    @staticmethod
    def image_gradient(I):
        """gradient kernel: central differences, one-sided at the borders; d1
        along columns, d2 along rows."""
        d1 = np.empty_like(I)
        d2 = np.empty_like(I)
        d1[:, :, 1:-1] = ((I[:, :, 2:] - I[:, :, :-2]).astype(f32) / f32(2)).astype(f32)
        d1[:, :, 0] = I[:, :, 1] - I[:, :, 0]
        d1[:, :, -1] = I[:, :, -1] - I[:, :, -2]
        d2[:, 1:-1, :] = ((I[:, 2:, :] - I[:, :-2, :]).astype(f32) / f32(2)).astype(f32)
        d2[:, 0, :] = I[:, 1, :] - I[:, 0, :]
        d2[:, -1, :] = I[:, -1, :] - I[:, -2, :]
        return d1, d2

    def regularization_gradient(self, dtau):
        """gradientRegularization + reduction7Dto6D + the two reductionsum passes
        (+ gradientJointAux): aux2[c][i][j], c = l + k * Cp for the control point
        in row k, column l, as the reference computes it:
          - dthetax / dthetax2 use dtau at the support pixel, times the
            derivative support splines (2 Dp S S', 2 Dp^2 S S'');
          - dthetat / dthetat2 use dtau at the transposed support corner
            (optimizer.cl:367-404 indexes dtaut without the offsets);
          - reduction7Dto6D sums dthetax over its last dimension with the
            stride getSpatialDimStride returns for dthetaallData: 17 floats
            (the header lookup assumes equal ranks, hostKernelFunctions.cl:195-233);
          - the frame reduction of reductionsum treats the frame axis as the
            outermost one, a sliding window of F consecutive (control point,
            frame) blocks (reductions.cl:91-111)."""
        g, F, Cp, dp = self.g, self.F, self.g.Cp, self.g.dp
        Dp = g.Dp
        dtaux, dtaux2, dtauxy, dtaut, dtaut2 = dtau
        S, S1, S2 = g.S
        l0, l1, l2, l3 = self.lam
        i_ = np.arange(dp)
        R = g.sup  # support start per control point (rows and columns alike)
        bbg = (S[:, None] * S[None, :]).astype(f32)                                 # BBg [i][j]
        b1g = [(f32(2 * Dp) * S[:, None] * S1[None, :]).astype(f32),
               (f32(2 * Dp) * S1[:, None] * S[None, :]).astype(f32)]
        b2g = [(f32(2 * Dp * Dp) * S[:, None] * S2[None, :]).astype(f32),
               (f32(2 * Dp * Dp) * S2[:, None] * S[None, :]).astype(f32)]
        b11g = (f32(2 * Dp * Dp) * S1[:, None] * S1[None, :]).astype(f32)
        # dtheta arrays in the reference's flat layouts: [p][d][l][k][f][i][j]
        # (elementwise products: gathered for every control point at once)
        RR = R[:, None] + i_[None, :]                                   # [cp][offset]
        rix, cix = RR[:, None, :, None], RR[None, :, None, :]           # (l, k, i, j)

        def at_support(a):  # a [..., F, N, N] -> [..., Cp(l), Cp(k), F, dp, dp]
            g_ = a[..., rix, cix]                                       # [..., F, Cp, Cp, dp, dp]
            nd = g_.ndim
            order = list(range(nd - 5)) + [nd - 4, nd - 3, nd - 5, nd - 2, nd - 1]
            return np.ascontiguousarray(g_.transpose(order))

        thx = (at_support(dtaux) * np.stack(b1g)[:, None, None, None, None]).astype(f32)
        thx2 = (at_support(dtaux2) * np.stack(b2g)[:, None, None, None, None]).astype(f32)
        thxy = (at_support(dtauxy) * b11g).astype(f32)
        # temporal terms: dtaut read at the transposed support corner [R[k]][R[l]]
        corner = lambda a: a[..., R[None, :], R[:, None]]               # [..., F, Cp(l), Cp(k)]
        c0, c2 = corner(dtaut), corner(dtaut2)                          # [d][f][l][k]
        c1, c21, c22 = np.roll(c0, -1, axis=1), np.roll(c2, -1, axis=1), np.roll(c2, -2, axis=1)
        t1 = (f32(2) * (c0 - c1).astype(f32)).astype(f32)
        t2 = (f32(2) * ((c2 - (f32(2) * c21).astype(f32)).astype(f32) + c22).astype(f32)).astype(f32)
        tht = (t1.transpose(0, 2, 3, 1)[..., None, None] * bbg).astype(f32)   # [d][l][k][f][i][j]
        tht2 = (t2.transpose(0, 2, 3, 1)[..., None, None] * bbg).astype(f32)
        n6 = thxy.size
        fx = thx.reshape(-1)
        fx2 = thx2.reshape(-1)
        s1 = ((f32(0) + fx[:n6]).astype(f32) + fx[17:n6 + 17]).astype(f32)
        s2 = ((f32(0) + fx2[:n6]).astype(f32) + fx2[17:n6 + 17]).astype(f32)
        aux = (l0 * s1).astype(f32)
        aux = (aux + (l1 * s2).astype(f32)).astype(f32)
        aux = (aux + (f32(l1 * f32(2)) * thxy.reshape(-1)).astype(f32)).astype(f32)
        aux = (aux + (l2 * tht.reshape(-1)).astype(f32)).astype(f32)
        aux = (aux + (l3 * tht2.reshape(-1)).astype(f32)).astype(f32)
        half = n6 // 2
        aux1 = ((f32(0) + aux[:half]).astype(f32) + aux[half:]).astype(f32)  # sum over d
        blk = dp * dp
        nblk = Cp * Cp
        aux2 = np.zeros(nblk * blk, f32)
        for t in range(F):
            aux2 = (aux2 + aux1[t * blk:(t + nblk) * blk]).astype(f32)
        return aux2.reshape(Cp, Cp, dp, dp)  # [l (Cp0 slot)][k (Cp1 slot)][i][j]

    def gradient(self, dx, dy, aux2):
        """gradientJoint + permutedV + the per-control-point loop of auxiliarMask,
        auxiliarCost, cost6DReduction, cost6D: dH [d][f][row cp][col cp].  The
        support sum runs in the reference's order (row offsets i summed for each
        column offset j, then the column sums), for every control point at once."""
        g, F, Cp, dp = self.g, self.F, self.g.Cp, self.g.dp
        S = g.S[0]
        bbg = (S[:, None] * S[None, :]).astype(f32)
        i_ = np.arange(dp)
        RR = g.sup[:, None] + i_[None, :]
        rix, cix = RR[:, None, :, None], RR[None, :, None, :]           # (kr, lc, i, j)
        mask = g.roi.T[rix, cix]                                        # [kr][lc][i][j]
        dyg = dy[:, rix, cix]                                           # [f][kr][lc][i][j]
        dH = np.zeros((2, F, Cp, Cp), f32)
        for d in range(2):
            dxg = dx[d][:, rix, cix]
            dv = (((dyg * dxg).astype(f32) * bbg).astype(f32) + aux2[None]).astype(f32)
            c1 = (dv * mask[None]).astype(f32)
            acc = np.zeros((F, Cp, Cp), f32)
            for jj in range(dp):
                col = np.zeros((F, Cp, Cp), f32)
                for ii in range(dp):
                    col = (col + c1[..., ii, jj]).astype(f32)
                acc = (acc + col).astype(f32)
            dH[d] = acc
        return dH

    def run(self, images, T_init=None):
        """T_init: the starting displacements (the reference's TData on a later
        motion iteration); the unregistered frames still give H[0] and the
        first dy, as optimizer() starts from a copy of the frames."""
        g, F, N = self.g, self.F, self.N
        x = np.asarray(images, np.complex64)
        oldmax = max(float(np.max(np.hypot(x[f].real, x[f].imag))) for f in range(F))
        factor = f32(f32(500) / f32(oldmax))
        I = (factor * np.hypot(x.real, x.imag).astype(f32)).astype(f32)
        d1, d2 = self.image_gradient(I)
        Cp = g.Cp
        T = np.zeros((2, F, Cp, Cp), f32) if T_init is None else np.array(T_init, f32).reshape(2, F, Cp, Cp)
        dtau = (np.zeros((2, 2, F, N, N), f32), np.zeros((2, 2, F, N, N), f32), np.zeros((2, F, N, N), f32),
                np.zeros((2, F, N, N), f32), np.zeros((2, F, N, N), f32))
        Iw = I.copy()
        V, mean = self.metric(Iw)
        H = [self.cost(V)]
        p2 = f32(self.et * f32(F * 2))
        p4 = f32(H[0] * self.eh)
        Wn = self.Wn
        fac = f32(2.0 / F)
        it = 1
        xn = None
        while True:
            xn = self.deform(T)
            dx = np.stack([self.warp(d1, xn), self.warp(d2, xn)])  # margin rectangle; elsewhere masked out
            dy = ((Iw - mean).astype(f32) * fac).astype(f32)
            aux2 = self.regularization_gradient(dtau)
            dH = self.gradient(dx, dy, aux2)
            mean4 = (_seqsum([dH[:, f] for f in range(F)]) / f32(F)).astype(f32)
            Dif = (Wn * (dH - mean4[:, None]).astype(f32)).astype(f32)
            T = (T - Dif).astype(f32)
            xn = self.deform(T)
            dtau = self.smoothness(T)
            Iw = self.warp(I, xn)
            V, mean = self.metric(Iw)
            if self.sum_lambda != 0:
                V = (V + self.smooth_metric(dtau).T).astype(f32)
            H.append(self.cost(V))
            Tdif = f32(np.sqrt(np.cumsum((Dif * Dif).astype(f32).reshape(-1), dtype=f32)[-1]))
            Hdif = f32(H[it - 1] - H[it])
            if self.flagW:
                # evolution(): (*Wn) * 1.2 in double, / 2 in float (GroupwiseRegistration.cpp:470-476)
                Wn = f32(float(Wn) * 1.2) if Hdif > 0 else f32(Wn / f32(2))
            if it == self.nmax or (Tdif < p2 and Hdif < p4):
                break
            it += 1
        return dict(T=T, xn=xn, H=np.array(H, f32), iterations=it, Wn=float(Wn))

    def smooth_metric(self, dtau):
        """sumLambdaMetric over the bounding box: the smoothness terms of the
        pixel at [r][c] of the dtau store (added at the transposed position)."""
        g, F = self.g, self.F
        dtaux, dtaux2, dtauxy, dtaut, dtaut2 = dtau
        l0, l1, l2, l3 = self.lam
        out = np.zeros((self.N, self.N), f32)
        rr, cc = np.meshgrid(g.box_rows, g.box_cols, indexing="ij")
        s = [np.zeros(rr.shape, f32) for _ in range(5)]
        for f in range(F):
            for d in range(2):
                s[2] = (s[2] + (f32(l1 * f32(2)) * (dtauxy[d, f][rr, cc] ** 2).astype(f32)).astype(f32)).astype(f32)
                s[3] = (s[3] + (l3 * (dtaut2[d, f][rr, cc] ** 2).astype(f32)).astype(f32)).astype(f32)
                s[4] = (s[4] + (l2 * (dtaut[d, f][rr, cc] ** 2).astype(f32)).astype(f32)).astype(f32)
                for p in range(2):
                    s[0] = (s[0] + (l0 * (dtaux[p, d, f][rr, cc] ** 2).astype(f32)).astype(f32)).astype(f32)
                    s[1] = (s[1] + (l1 * (dtaux2[p, d, f][rr, cc] ** 2).astype(f32)).astype(f32)).astype(f32)
        tot = _seqsum(s)
        out[rr, cc] = tot
        return out
