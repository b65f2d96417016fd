"""D3Q19 discrete velocity set with the H10 Hermite moment space
(jyulb/D3Q19.pyx, jyulb/D3Q19.pxd).

``D3Q19_H10`` carries the reference's tables under the same attribute names.
Its moment maps and forward-Euler updates are NumPy functions over arrays of
shape (19, ...) (any trailing node shape); on the GPU the same physics runs
inside the fused step kernels.  Moments are sums over lattice vectors, as in
the reference.
"""
from __future__ import annotations

import numpy as np

from .defs import FACE_1X, FACE_X1, FACE_1Y, FACE_Y1, FACE_1Z, FACE_Z1

# lattice-vector enumeration (jyulb/D3Q19.pxd:59-79)
L_1I_1J_K0, L_1I_J0_1K, L_1I_J0_K0, L_1I_J0_K1, L_1I_J1_K0 = 0, 1, 2, 3, 4
L_I0_1J_1K, L_I0_1J_K0, L_I0_1J_K1 = 5, 6, 7
L_I0_J0_1K, L_I0_J0_K0, L_I0_J0_K1 = 8, 9, 10
L_I0_J1_1K, L_I0_J1_K0, L_I0_J1_K1 = 11, 12, 13
L_I1_1J_K0, L_I1_J0_1K, L_I1_J0_K0, L_I1_J0_K1, L_I1_J1_K0 = 14, 15, 16, 17, 18
LVECS = 19

# Hermite moments (jyulb/D3Q19.pxd:85-96)
H0, H1_X, H1_Y, H1_Z, H2_XX, H2_XY, H2_XZ, H2_YY, H2_YZ, H2_ZZ = range(10)
HMOMS = 10

LI = np.array([-1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1], dtype=np.int32)
LJ = np.array([-1, 0, 0, 0, 1, -1, -1, -1, 0, 0, 0, 1, 1, 1, -1, 0, 0, 0, 1], dtype=np.int32)
LK = np.array([0, -1, 0, 1, 0, -1, 0, 1, -1, 0, 1, -1, 0, 1, 0, -1, 0, 1, 0], dtype=np.int32)


class D3Q19_H10:
    """Tables of the D3Q19 velocity set (jyulb/D3Q19.pyx:66-275)."""

    def __init__(self):
        self.B1 = np.array([1.0, 0.0, 0.0])
        self.B2 = np.array([0.0, 1.0, 0.0])
        self.B3 = np.array([0.0, 0.0, 1.0])
        self.AS = np.sqrt(3.0)
        self.AS2 = 3.0
        self.AS4 = 9.0
        self.INV_AS = 1.0 / self.AS
        self.INV_AS2 = 1.0 / 3.0
        self.INV_AS4 = 1.0 / 9.0
        self.W0, self.W1, self.W2 = 12.0 / 36.0, 2.0 / 36.0, 1.0 / 36.0
        self.LI, self.LJ, self.LK = LI.copy(), LJ.copy(), LK.copy()
        self.LX = LI.astype(np.float64)
        self.LY = LJ.astype(np.float64)
        self.LZ = LK.astype(np.float64)
        self.OPP_LVEC = np.array([18 - l for l in range(LVECS)], dtype=np.uint8)
        nnz = (LI != 0).astype(int) + (LJ != 0) + (LK != 0)
        self.LW = np.where(nnz == 0, self.W0, np.where(nnz == 1, self.W1, self.W2))
        self.FDIR_LVECS = 5
        self.FDIR_LVEC = np.zeros((6, 5), dtype=np.int32)
        for face, (comp, sign) in enumerate([(LI, -1), (LI, 1), (LJ, -1), (LJ, 1), (LK, -1), (LK, 1)]):
            self.FDIR_LVEC[face] = np.nonzero(comp == sign)[0]
        self.LRANGE = 1
        self.LSPAN = 3
        lx, ly, lz = self.LX, self.LY, self.LZ
        self.HPOL2_XX = lx * lx - self.INV_AS2
        self.HPOL2_XY = lx * ly
        self.HPOL2_XZ = lx * lz
        self.HPOL2_YY = ly * ly - self.INV_AS2
        self.HPOL2_YZ = ly * lz
        self.HPOL2_ZZ = lz * lz - self.INV_AS2
        self.K1_X = self.AS2 * self.LW * lx
        self.K1_Y = self.AS2 * self.LW * ly
        self.K1_Z = self.AS2 * self.LW * lz
        self.K2_XX = 0.5 * self.AS4 * self.LW * self.HPOL2_XX
        self.K2_XY = 0.5 * self.AS4 * self.LW * self.HPOL2_XY
        self.K2_XZ = 0.5 * self.AS4 * self.LW * self.HPOL2_XZ
        self.K2_YY = 0.5 * self.AS4 * self.LW * self.HPOL2_YY
        self.K2_YZ = 0.5 * self.AS4 * self.LW * self.HPOL2_YZ
        self.K2_ZZ = 0.5 * self.AS4 * self.LW * self.HPOL2_ZZ

    # -- moments (jyulb/D3Q19.pyx:283-452) -------------------------------
    def f_to_den(self, f):
        """Density: the sum of all 19 populations.  (The reference's
        ``f_to_den``, jyulb/D3Q19.pyx:283-301, adds three populations twice and
        omits three; it is never called there.  This returns the true sum.)"""
        return np.sum(f, axis=0)

    def f_to_den_mom(self, f):
        den = np.sum(f, axis=0)
        mom = np.stack([np.tensordot(self.LX, f, 1), np.tensordot(self.LY, f, 1),
                        np.tensordot(self.LZ, f, 1)])
        return den, mom

    def f_to_den_vel(self, f):
        den, mom = self.f_to_den_mom(f)
        return den, mom / den

    def f_to_h(self, f):
        den, mom = self.f_to_den_mom(f)
        h = np.empty((HMOMS,) + np.shape(den))
        h[H0] = den
        h[H1_X:H1_Z + 1] = mom
        lx, ly, lz = self.LX, self.LY, self.LZ
        h[H2_XX] = np.tensordot(lx * lx, f, 1) - self.INV_AS2 * den
        h[H2_XY] = np.tensordot(lx * ly, f, 1)
        h[H2_XZ] = np.tensordot(lx * lz, f, 1)
        h[H2_YY] = np.tensordot(ly * ly, f, 1) - self.INV_AS2 * den
        h[H2_YZ] = np.tensordot(ly * lz, f, 1)
        h[H2_ZZ] = np.tensordot(lz * lz, f, 1) - self.INV_AS2 * den
        return h

    # -- projections (jyulb/D3Q19.pyx:460-630) ---------------------------
    def h_to_f(self, h):
        """Kinetic projection f_l = w_l (h0 + 3 c.h1 + 4.5 H2(c):h2)."""
        h = np.asarray(h, dtype=np.float64)
        K = np.stack([self.LW, self.K1_X, self.K1_Y, self.K1_Z, self.K2_XX, 2 * self.K2_XY,
                      2 * self.K2_XZ, self.K2_YY, 2 * self.K2_YZ, self.K2_ZZ], axis=1)
        return np.tensordot(K, h, 1)

    def add_h_to_f(self, h, f):
        f += self.h_to_f(h)
        return f

    def den_vel_to_heq(self, den, vel):
        den = np.asarray(den, dtype=np.float64)
        vel = np.asarray(vel, dtype=np.float64)
        j = den * vel
        return np.stack([den, j[0], j[1], j[2], j[0] * vel[0], j[0] * vel[1], j[0] * vel[2],
                         j[1] * vel[1], j[1] * vel[2], j[2] * vel[2]])

    def eq(self, den, vel):
        return self.h_to_f(self.den_vel_to_heq(den, vel))

    # -- forward-Euler updates (jyulb/D3Q19.pyx:655-940) ------------------
    def _force(self, h, c1, c2, acc, den, j):
        a = np.asarray(acc, dtype=np.float64).reshape((3,) + (1,) * (np.ndim(den)))
        h[H1_X:H1_Z + 1] += c1 * a * den
        h[H2_XX] += 2.0 * c2 * a[0] * j[0]
        h[H2_XY] += c2 * (a[0] * j[1] + a[1] * j[0])
        h[H2_XZ] += c2 * (a[0] * j[2] + a[2] * j[0])
        h[H2_YY] += 2.0 * c2 * a[1] * j[1]
        h[H2_YZ] += c2 * (a[1] * j[2] + a[2] * j[1])
        h[H2_ZZ] += 2.0 * c2 * a[2] * j[2]

    def forw_euler_BGK(self, f, acc, prm):
        """Returns (den, vel, f_post); vel = j/den + acc/2."""
        w = prm[0]
        den, vel = self.f_to_den_vel(f)
        a = np.asarray(acc, dtype=np.float64).reshape((3,) + (1,) * np.ndim(den))
        vel = vel + 0.5 * a
        h = w * self.den_vel_to_heq(den, vel)
        self._force(h, 1.0 - 0.5 * w, 1.0 - 0.5 * w, acc, den, den * vel)
        return den, vel, (1.0 - w) * f + self.h_to_f(h)

    def forw_euler_TRT(self, f, acc, prm):
        we, wo = prm[0], prm[1]
        den, vel = self.f_to_den_vel(f)
        a = np.asarray(acc, dtype=np.float64).reshape((3,) + (1,) * np.ndim(den))
        vel = vel + 0.5 * a
        h = self.den_vel_to_heq(den, vel)
        h[H0] *= we
        h[H1_X:H1_Z + 1] *= wo
        h[H2_XX:] *= we
        self._force(h, 1.0 - 0.5 * wo, 1.0 - 0.5 * we, acc, den, den * vel)
        c3, c4 = 1.0 - 0.5 * (we + wo), 0.5 * (we - wo)
        fo = f[::-1]
        g = c3 * f - c4 * fo
        g[9] = (1.0 - we) * f[9]
        return den, vel, g + self.h_to_f(h)

    def forw_euler_regul(self, f, acc, prm):
        w = prm[0]
        h = self.f_to_h(f)
        den = h[H0]
        a = np.asarray(acc, dtype=np.float64).reshape((3,) + (1,) * np.ndim(den))
        j = h[H1_X:H1_Z + 1] + 0.5 * a * den
        vel = j / den
        he = self.den_vel_to_heq(den, vel)
        h = (1.0 - w) * h + w * he
        self._force(h, 1.0 - 0.5 * w, 1.0 - 0.5 * w, acc, den, j)
        return den, vel, self.h_to_f(h)
