"""The raster stage's conservative row spans (raster_kernels.cu: span_edges / span_code), restated
with the same float32 operations, never exclude a pixel that has a covered sample.

For each tile row r and edge i with A != 0 the kernel bounds the columns by the crossing
t = (E(0, 256r) + max_k(A sx_k + B sy_k)) * (-1 / (256 A)), clamped to [-2, TS + 1], and takes
ceil(t - 2^-10) as the first column (A > 0) or floor(t + 2^-10) as the last (A < 0); an edge with
A == 0 empties the row when its largest value is negative.  Edge functions follow the 16.8
fixed-point set-up: E_i = A_i (x - X_j) + B_i (y - Y_j) - bias, covered when all three are >= 0."""
import numpy as np

# 4x pattern in 1/256 pixel (the standard D3D positions)
SX = np.array([96, 224, 32, 160])
SY = np.array([32, 96, 160, 224])
TS = 16
EPS = np.float32(1.0 / 1024)


def edges(V):
    A, B, C = [], [], []
    for i in range(3):
        j, k = (i + 1) % 3, (i + 2) % 3
        a = int(V[j, 1] - V[k, 1])
        b = int(V[k, 0] - V[j, 0])
        bias = 0 if (a > 0 or (a == 0 and b > 0)) else 1
        A.append(a)
        B.append(b)
        C.append(-a * int(V[j, 0]) - b * int(V[j, 1]) - bias)
    return A, B, C


def spans(A, B, C):
    out = []
    for r in range(TS):
        lo, hi, empty = 0, TS - 1, False
        for i in range(3):
            m = max(A[i] * int(SX[k]) + B[i] * int(SY[k]) for k in range(4))
            b = C[i] + m + B[i] * 256 * r
            rcp = np.float32(-1.0) / (np.float32(256.0) * np.float32(A[i])) if A[i] != 0 else np.float32(0)
            t = min(max(np.float32(b) * rcp, np.float32(-2.0)), np.float32(TS + 1))
            if A[i] > 0:
                lo = max(lo, int(np.ceil(np.float32(t - EPS))))
            elif A[i] < 0:
                hi = min(hi, int(np.floor(np.float32(t + EPS))))
            else:
                empty |= b < 0
        out.append(None if empty or lo > hi else (lo, hi))
    return out


def coverage(A, B, C):
    qx, qy = np.meshgrid(np.arange(TS), np.arange(TS))
    cov = np.zeros((TS, TS), bool)
    for k in range(4):
        x = qx * 256 + SX[k]
        y = qy * 256 + SY[k]
        ok = np.ones((TS, TS), bool)
        for i in range(3):
            ok &= (A[i] * x + B[i] * y + C[i]) >= 0
        cov |= ok
    return cov


def _triangles(rng, n):
    for _ in range(n):
        if rng.uniform() < 0.5:  # slivers like the benchmark's soup
            L = 4 * np.exp(rng.normal())
            h = 0.2 * L * rng.uniform(0.5, 1.5)
            th = rng.uniform(0, 2 * np.pi)
            ex, ey = np.array([np.cos(th), np.sin(th)]), np.array([-np.sin(th), np.cos(th)])
            c = rng.uniform(0, 16, 2)
            P = np.array([c - 0.5 * L * ex - h * ey / 3, c + 0.5 * L * ex - h * ey / 3,
                          c + rng.uniform(-0.5, 0.5) * L * ex + 2 * h / 3 * ey])
        else:  # anything from sub-pixel to much larger than the tile
            P = rng.uniform(-20, 36, 2) + rng.normal(size=(3, 2)) * 10 ** rng.uniform(-0.5, 3)
        V = np.round(P * 256).astype(np.int64)
        ar = (V[1, 0] - V[0, 0]) * (V[2, 1] - V[0, 1]) - (V[2, 0] - V[0, 0]) * (V[1, 1] - V[0, 1])
        if ar == 0:
            continue
        yield V if ar > 0 else V[[0, 2, 1]]


def test_row_spans_are_conservative_and_tight():
    rng = np.random.default_rng(7)
    span_px = cov_px = 0
    for V in _triangles(rng, 600):
        A, B, C = edges(V)
        cov = coverage(A, B, C)
        sp = spans(A, B, C)
        for r in range(TS):
            xs = np.nonzero(cov[r])[0]
            if len(xs):
                assert sp[r] is not None and sp[r][0] <= xs.min() and xs.max() <= sp[r][1], (V, r, sp[r], xs)
            if sp[r] is not None:
                span_px += sp[r][1] - sp[r][0] + 1
        cov_px += int(cov.sum())
    # the spans are close to the covered set (a bbox would be several times larger for slivers)
    assert cov_px > 0 and span_px < 1.5 * cov_px, (span_px, cov_px)
