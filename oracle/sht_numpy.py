"""Independent small-truncation transform oracle -- TEST INFRASTRUCTURE ONLY.

A second restatement of the src/shtns.f90 transform contract, written with
different machinery from gd_oracle.cpp so the two cross-check each other:
Gauss nodes from numpy's ``leggauss``, associated Legendre values from
scipy's ``lpmv`` with explicit normalisation, and explicit DFT matrices in
place of an FFT.  Only practical for T <= ~60.

Conventions (src/shtns.f90:51-53, :110, :149-150): orthonormal harmonics
(integral of |Y|^2 over the sphere = 1) without Condon-Shortley phase;
m-major triangular order; real fields, m > 0 coefficients stand for the
(+m, -m) pair; latitudes north to south.  getuv / getvrtdivspec / getgrad
follow the physical contract of src/shtns.f90:233-352: u eastward, v
northward, vrt = k.curl(V), div = div(V), grad = (df/(a cos dlambda),
df/(a dphi)).
"""
import numpy as np
from numpy.polynomial.legendre import leggauss
from scipy.special import gammaln, lpmv


class ShtNumpy:
    def __init__(self, T, nlon, nlat, rsphere=6.3712e6):
        self.T, self.nlon, self.nlat, self.a = T, nlon, nlat, float(rsphere)
        x, w = leggauss(nlat)
        self.mu = x[::-1].copy()
        self.w = w[::-1].copy()
        self.W = 2 * np.pi * self.w
        self.phi = np.arcsin(self.mu)
        self.cos = np.sqrt(1 - self.mu ** 2)
        self.lam = 2 * np.pi * np.arange(nlon) / nlon
        self.deg = np.concatenate([np.arange(m, T + 1) for m in range(T + 1)])
        self.order = np.concatenate([np.full(T - m + 1, m) for m in range(T + 1)])
        self.nlm = self.deg.size
        P = np.zeros((self.nlm, nlat))
        H = np.zeros((self.nlm, nlat))
        for k, (n, m) in enumerate(zip(self.deg, self.order)):
            norm = np.sqrt((2 * n + 1) / (4 * np.pi) * np.exp(gammaln(n - m + 1) - gammaln(n + m + 1)))
            # lpmv carries the Condon-Shortley phase (-1)^m; remove it.
            P[k] = norm * (-1.0) ** m * lpmv(m, n, self.mu)
            # (1-x^2) dP_n^m/dx = -n x P_n^m + (n+m) P_{n-1}^m, dP/dphi = cos dP/dx
            pnm1 = (-1.0) ** m * lpmv(m, n - 1, self.mu) if n - 1 >= m else 0.0 * self.mu
            H[k] = norm * (-n * self.mu * (-1.0) ** m * lpmv(m, n, self.mu) + (n + m) * pnm1) / self.cos
        self.P, self.H = P, H
        ms = np.arange(T + 1)
        self.E = np.exp(1j * np.outer(ms, self.lam))  # [m, i]

    def _block(self, tab, a):
        """F[m, j] = sum_n tab[nm, j] a[nm]."""
        F = np.zeros((self.T + 1, self.nlat), np.complex128)
        np.add.at(F, self.order, tab * a[:, None])
        return F

    def _f2g(self, F):
        g = np.real(F[0])[:, None] * np.ones(self.nlon)
        g = g + 2 * np.real(F[1:].T @ self.E[1:])
        return g

    def _g2f(self, g):
        return (g @ np.conj(self.E).T).T / self.nlon  # [m, j]

    def _anal(self, tab, F):
        return np.sum(tab * (self.W * F[self.order]), axis=1)

    def _imcos(self, F):
        return F * (1j * np.arange(self.T + 1)[:, None] / self.cos[None, :])

    def spectogrd(self, a):
        return self._f2g(self._block(self.P, a))

    def grdtospec(self, g):
        return self._anal(self.P, self._g2f(g))

    def getuv(self, vrt, div):
        il = np.zeros(self.nlm)
        il[1:] = -1.0 / (self.deg[1:] * (self.deg[1:] + 1.0))
        s = self.a * il * vrt
        c = self.a * il * div
        U = -self._block(self.H, s) + self._imcos(self._block(self.P, c))
        V = self._imcos(self._block(self.P, s)) + self._block(self.H, c)
        return self._f2g(U), self._f2g(V)

    def getvrtdivspec(self, u, v):
        U, V = self._g2f(u), self._g2f(v)
        vrt = (self._anal(self.P, self._imcos(V)) + self._anal(self.H, U)) / self.a
        div = (self._anal(self.P, self._imcos(U)) - self._anal(self.H, V)) / self.a
        return vrt, div

    def getgrad(self, f):
        gx = self._f2g(self._imcos(self._block(self.P, f))) / self.a
        gy = self._f2g(self._block(self.H, f)) / self.a
        return gx, gy
