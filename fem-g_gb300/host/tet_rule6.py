"""Parameters of the 24-point degree-6 tetrahedral rule used for "Gauss6" on
tetrahedra (host/refelem.cpp, keastTet6): three orbits of barycentric
(a, a, a, 1 - 3a) and one of (a, a, b, 1 - 2a - b), the orbit structure of
Keast's rule 6 (Comput. Methods Appl. Mech. Eng. 55, 1986). Solves the moment
equations (every monomial u^i v^j w^k, i + j + k <= 6, integrated exactly over
the reference tetrahedron of volume 1/6) from a start near the published
values, by Gauss-Newton in 40-digit arithmetic, and prints the nine
parameters (a1, w1, a2, w2, a3, w3, a, b, w)."""
import itertools

import mpmath as mp

mp.mp.dps = 40
MONOMIALS = [(i, j, k) for i in range(7) for j in range(7) for k in range(7) if i + j + k <= 6]
EXACT = [mp.factorial(i) * mp.factorial(j) * mp.factorial(k) / mp.factorial(i + j + k + 3) for i, j, k in MONOMIALS]


def points(x):
    a1, w1, a2, w2, a3, w3, a, b, w = x
    out = []
    for aa, ww in ((a1, w1), (a2, w2), (a3, w3)):
        for k in range(4):
            lam = [aa] * 4
            lam[k] = 1 - 3 * aa
            out.append((lam, ww))
    for i, j in itertools.permutations(range(4), 2):
        lam = [a] * 4
        lam[i] = b
        lam[j] = 1 - 2 * a - b
        out.append((lam, w))
    return out


def residual(x):
    pts = points(x)
    return [sum(w * l[1] ** i * l[2] ** j * l[3] ** k for l, w in pts) - e for (i, j, k), e in zip(MONOMIALS, EXACT)]


def solve(x0, steps=10):
    x = [mp.mpf(v) for v in x0]
    h = mp.mpf("1e-25")
    for _ in range(steps):
        f = mp.matrix(residual(x))
        J = mp.matrix(len(MONOMIALS), 9)
        for c in range(9):
            xp = list(x)
            xp[c] += h
            fp = residual(xp)
            for r in range(len(MONOMIALS)):
                J[r, c] = (fp[r] - f[r]) / h
        dx = mp.lu_solve(J.T * J, J.T * f)
        x = [x[c] - dx[c] for c in range(9)]
    return x, max(abs(v) for v in residual(x))


if __name__ == "__main__":
    start = ["0.0407", "0.00168", "0.2146", "0.00665", "0.3223", "0.00923", "0.0637", "0.603", "0.00804"]
    x, res = solve(start)
    for v in x:
        print(mp.nstr(v, 25))
    print("max moment residual", mp.nstr(res, 3))
