"""Coefficients of the kernels' double-precision sine and cosine.

sin r = r + r^3 P(r^2) and cos r = 1 + r^2 Q(r^2) on |r| <= pi/4, with P and
Q of degree 5, fitted as near-minimax polynomials of the
weighted (relative) error by Lawson's algorithm (iteratively reweighted least
squares; C. L. Lawson, 1961) at 400 Chebyshev nodes in z = r^2, in 60-digit
arithmetic (mpmath), then rounded to double.  Prints the coefficients, lowest
degree first, as C hex literals; ode_solver.cuh (sincos_cw) and the oracle
(sincos_dev) hold the printed values.

Usage: python gen_sincos.py
"""
import mpmath as mp

mp.mp.dps = 60
ZMAX = (mp.pi / 4) ** 2


def lawson_fit(fun, weight, deg, n=400, iters=30):
    nodes = [ZMAX * (1 - mp.cos(mp.pi * (i + mp.mpf(1) / 2) / n)) / 2 for i in range(n)]
    w = [weight(z) for z in nodes]
    lam = [mp.mpf(1)] * n
    for _ in range(iters):
        A = mp.matrix(n, deg + 1)
        b = mp.matrix(n, 1)
        for i, z in enumerate(nodes):
            s = mp.sqrt(lam[i]) * w[i]
            for j in range(deg + 1):
                A[i, j] = s * z ** j
            b[i] = s * fun(z)
        c = mp.lu_solve(A.T * A, A.T * b)
        err = [abs(w[i] * (sum(c[j] * nodes[i] ** j for j in range(deg + 1)) - fun(nodes[i]))) for i in range(n)]
        m = max(err)
        lam = [lam[i] * (err[i] / m + mp.mpf("1e-3")) for i in range(n)]
    return [c[j] for j in range(deg + 1)], m


def main():
    fs = lambda z: (mp.sin(mp.sqrt(z)) - mp.sqrt(z)) / (z * mp.sqrt(z))
    fc = lambda z: (mp.cos(mp.sqrt(z)) - 1) / z
    ws = lambda z: z / (mp.sin(mp.sqrt(z)) / mp.sqrt(z))   # relative error of sin r per unit error of P
    wc = lambda z: z / mp.cos(mp.sqrt(z))                  # relative error of cos r per unit error of Q
    for name, f, w, deg in (("P (sin)", fs, ws, 5), ("Q (cos)", fc, wc, 5)):
        c, m = lawson_fit(f, w, deg)
        print("%s: max relative error %.2e" % (name, float(m)))
        print("  " + ", ".join(float(x).hex() for x in c))


if __name__ == "__main__":
    main()
