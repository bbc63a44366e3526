"""ORACLE — test infrastructure only.

An independent pure-Python restatement of src/decomp/lu.rs:104-168 (factor),
:224-232 (det) and :237-278 (solve), src/matrix/mod.rs:957-980 (Mul),
src/decomp/cholesky.rs:56-145 (Cholesky factor and solve) and
src/decomp/qr.rs:26-235 (QR factor, Q and solve), written
with plain Python floats (IEEE binary64, no fused multiply-add) and lists. It is
slow and meant only for small matrices: it cross-checks the C restatement.
"""


def lu_factor(a):
    m = len(a)
    n = len(a[0])
    lu = [float(v) for row in a for v in row]
    piv = list(range(m))
    pos = True
    for j in range(n):
        for i in range(m):
            s = 0.0
            for k in range(min(i, j)):
                s = s + lu[i * n + k] * lu[k * n + j]
            lu[i * n + j] = lu[i * n + j] - s
        p = j
        for i in range(j + 1, m):
            if abs(lu[i * n + j]) > abs(lu[p * n + j]):
                p = i
        if p != j:
            for k in range(n):
                lu[p * n + k], lu[j * n + k] = lu[j * n + k], lu[p * n + k]
            piv[p], piv[j] = piv[j], piv[p]
            pos = not pos
        if j < m and lu[j * n + j] != 0.0:
            for i in range(j + 1, m):
                lu[i * n + j] = lu[i * n + j] / lu[j * n + j]
    return lu, piv, pos


def det(lu, n, pos):
    d = 1.0 if pos else -1.0
    for j in range(n):
        d = d * lu[j * n + j]
    return d


def solve(lu, m, n, piv, b, nx):
    for j in range(n):
        if lu[j * n + j] == 0.0:
            return None
    x = [b[piv[i] * nx + j] for i in range(m) for j in range(nx)]
    for k in range(n):
        for i in range(k + 1, n):
            for j in range(nx):
                x[i * nx + j] = x[i * nx + j] - x[k * nx + j] * lu[i * n + k]
    for k in range(n - 1, -1, -1):
        for j in range(nx):
            x[k * nx + j] = x[k * nx + j] / lu[k * n + k]
        for i in range(k):
            for j in range(nx):
                x[i * nx + j] = x[i * nx + j] - x[k * nx + j] * lu[i * n + k]
    return x


def matmul(a, b):
    m, k, n = len(a), len(b), len(b[0])
    out = []
    for r in range(m):
        row = []
        for c in range(n):
            res = 0.0
            for idx in range(k):
                res = res + a[r][idx] * b[idx][c]
            row.append(res)
        out.append(row)
    return out


def chol_new(a):
    """src/decomp/cholesky.rs:56-111 with Python floats: the n*n factor as a flat
    list, or None (non-square, non-symmetric, not positive definite)."""
    import math
    if len(a) != len(a[0]):
        return None
    n = len(a)
    l = [0.0] * (n * n)
    for j in range(n):
        d = 0.0
        for k in range(j):
            s = 0.0
            for i in range(k):
                s = s + l[k * n + i] * l[j * n + i]
            s = (float(a[j][k]) - s) / l[k * n + k]
            l[j * n + k] = s
            d = d + s * s
            if float(a[k][j]) != float(a[j][k]):
                return None
        d = float(a[j][j]) - d
        if d <= 0.0:
            return None
        l[j * n + j] = math.sqrt(d)
        for k in range(j + 1, n):
            l[j * n + k] = 0.0
    return l


def chol_solve(l, n, b, nx):
    """src/decomp/cholesky.rs:116-145 (b flat, row-major n x nx)."""
    x = [float(v) for v in b]
    for k in range(n):
        for j in range(nx):
            for i in range(k):
                x[k * nx + j] = x[k * nx + j] - x[i * nx + j] * l[k * n + i]
            x[k * nx + j] = x[k * nx + j] / l[k * n + k]
    for k in range(n - 1, -1, -1):
        for j in range(nx):
            for i in range(k + 1, n):
                x[k * nx + j] = x[k * nx + j] - x[i * nx + j] * l[i * n + k]
            x[k * nx + j] = x[k * nx + j] / l[k * n + k]
    return x


def qr_new(a):
    """src/decomp/qr.rs:26-105 with Python floats: (qr flat m*n, rdiag)."""
    import math
    m, n = len(a), len(a[0])
    q = [float(v) for row in a for v in row]
    rd = []
    for minor in range(min(m, n)):
        x = 0.0
        for i in range(minor, m):
            c = q[i * n + minor]
            x = x + c * c
        a0 = -math.sqrt(x) if q[minor * n + minor] > 0.0 else math.sqrt(x)
        rd.append(a0)
        if a0 != 0.0:
            q[minor * n + minor] = q[minor * n + minor] - a0
            for col in range(minor + 1, n):
                d = 0.0
                for row in range(minor, m):
                    d = d + q[row * n + minor] * q[row * n + col]
                f = d / (a0 * q[minor * n + minor])
                for row in range(minor, m):
                    q[row * n + col] = q[row * n + col] + f * q[row * n + minor]
    return q, rd


def qr_get_q(q, rd, m, n):
    """src/decomp/qr.rs:151-194 (m x m, flat)."""
    out = [0.0] * (m * m)
    for k in range(min(m, n)):
        out[k * m + k] = 1.0
    for k in range(min(m, n) - 1, -1, -1):
        if q[k * n + k] != 0.0:
            for col in range(k, m):
                d = 0.0
                for row in range(k, m):
                    d = d + q[row * n + k] * out[row * m + col]
                f = d / (rd[k] * q[k * n + k])
                for row in range(k, m):
                    out[row * m + col] = out[row * m + col] + f * q[row * n + k]
    return out


def qr_solve(q, rd, m, n, b, nx):
    """src/decomp/qr.rs:211-235 for a square, full-rank factor (b flat m x nx)."""
    x = [float(v) for v in b]
    for k in range(n):
        for j in range(nx):
            s = 0.0
            for i in range(k, m):
                s = s + q[i * n + k] * x[i * nx + j]
            s = -s / q[k * n + k]
            for i in range(k, m):
                x[i * nx + j] = x[i * nx + j] + s * q[i * n + k]
    for k in range(n - 1, -1, -1):
        for j in range(nx):
            x[k * nx + j] = x[k * nx + j] / rd[k]
        for i in range(k):
            for j in range(nx):
                x[i * nx + j] = x[i * nx + j] - x[k * nx + j] * q[i * n + k]
    return x
