"""The unfused path's column stage, restated on the CPU.

`k_plain_cols_fwd` (csrc/plain_cols.cu) gives each CTA C left columns of one
pair of patches and their mirrors c -> (P - c) mod P; group 0 also holds the
self-mirror column P / 2.  Each column of length P = 16 L1 is transformed in
shared memory by an in-place four-step in a padded layout (y = n1 + L1 n2 at
n1 + Q n2, Q odd), natural -> permuted forward (X[k2 + 16 k1] at Q k2 + k1) and
permuted -> natural inverse.  The pair's two patch spectra come from Z(k) and
Z(-k), and the PSF spectra from the stored half plane kx <= P / 2.

Here the same index plan runs in numpy at small sides (the kernel is built for
L1 in {10, 12, 16, 20, 24, 32}; the plan does not depend on L1).  It must cover
every column once, and it must give the column transform, the products
A Ha + iB Hb and the inverse column transform of numpy's FFTs.
"""
import numpy as np
import pytest


class Plan:
    def __init__(self, L1, C):
        self.L1, self.C = L1, C
        self.P = 16 * L1
        self.Q = L1 + 1 if L1 % 2 == 0 else L1 + 2
        self.CP = 16 * self.Q + 1
        self.NC = 2 * C
        self.G = (self.P // 2) // C
        self.tw = np.exp(-2j * np.pi * np.arange(self.P) / self.P)

    def pos(self, y):
        return y + (y // self.L1) * (self.Q - self.L1)

    def spos(self, k):
        return self.Q * (k & 15) + (k >> 4)

    def col(self, s, g):
        if s < self.C:
            return g * self.C + s
        t = g * self.C + (s - self.C)
        return self.P // 2 if t == 0 else self.P - t

    def mirror(self, s, g):
        if g == 0 and s in (0, self.C):
            return s
        return s + self.C if s < self.C else s - self.C

    def forward(self, buf):
        L1, Q, CP = self.L1, self.Q, self.CP
        for s in range(self.NC):
            for n1 in range(L1):
                idx = [s * CP + n1 + Q * n2 for n2 in range(16)]
                v = np.fft.fft(buf[idx])
                buf[idx] = v * np.array([self.tw[n1 * k2] for k2 in range(16)])
            for k2 in range(16):
                idx = [s * CP + Q * k2 + n1 for n1 in range(L1)]
                buf[idx] = np.fft.fft(buf[idx])

    def inverse(self, buf):
        L1, Q, CP = self.L1, self.Q, self.CP
        for s in range(self.NC):
            for k2 in range(16):
                idx = [s * CP + Q * k2 + k1 for k1 in range(L1)]
                v = np.fft.ifft(buf[idx]) * L1
                buf[idx] = v * np.conj([self.tw[n1 * k2] for n1 in range(L1)])
            for n1 in range(L1):
                idx = [s * CP + n1 + Q * n2 for n2 in range(16)]
                buf[idx] = np.fft.ifft(buf[idx]) * 16


def hermitian_full(H, P):
    """The full P x P spectrum from the stored half plane kx <= P / 2."""
    F = np.empty((P, P), complex)
    for ky in range(P):
        for kx in range(P):
            F[ky, kx] = H[ky, kx] if kx <= P // 2 else np.conj(H[(P - ky) % P, P - kx])
    return F


@pytest.mark.parametrize("L1,C", [(2, 1), (2, 4), (3, 2), (4, 8)])
def test_groups_cover_every_column_once_and_hold_their_mirrors(L1, C):
    pl = Plan(L1, C)
    cols = sorted(pl.col(s, g) for g in range(pl.G) for s in range(pl.NC))
    assert cols == list(range(pl.P))
    for g in range(pl.G):
        for s in range(pl.NC):
            assert pl.col(pl.mirror(s, g), g) == (pl.P - pl.col(s, g)) % pl.P
    # the padded places of the natural and the permuted orders are the same set
    # (the kernel stores either through pos)
    assert sorted(map(pl.pos, range(pl.P))) == sorted(map(pl.spos, range(pl.P)))
    assert (pl.NC - 1) * pl.CP + max(map(pl.pos, range(pl.P))) < pl.NC * pl.CP


@pytest.mark.parametrize("L1,C", [(2, 1), (3, 2), (4, 4)])
def test_forward_stage_matches_numpy(L1, C):
    pl = Plan(L1, C)
    P = pl.P
    rng = np.random.default_rng(L1 * 10 + C)
    Z = rng.normal(size=(P, P)) + 1j * rng.normal(size=(P, P))  # row-transformed pair
    Ha = rng.normal(size=(P, P // 2 + 1)) + 1j * rng.normal(size=(P, P // 2 + 1))
    Hb = rng.normal(size=(P, P // 2 + 1)) + 1j * rng.normal(size=(P, P // 2 + 1))
    # numpy: column FFT, the two patches' spectra, the products, inverse column FFT
    X = np.fft.fft(Z, axis=0)
    neg = (-np.arange(P)) % P
    Xm = np.conj(X[neg][:, neg])
    W = (X + Xm) / 2 * hermitian_full(Ha, P) + (X - Xm) / 2 * hermitian_full(Hb, P)
    ref = np.fft.ifft(W, axis=0) * P
    out = np.zeros((P, P), complex)
    for g in range(pl.G):
        bz = np.zeros(pl.NC * pl.CP, complex)
        for s in range(pl.NC):
            for y in range(P):
                bz[s * pl.CP + pl.pos(y)] = Z[y, pl.col(s, g)]
        pl.forward(bz)
        for s in range(pl.NC):  # the forward leaves X[k] at spos(k)
            got = [bz[s * pl.CP + pl.spos(k)] for k in range(P)]
            np.testing.assert_allclose(got, X[:, pl.col(s, g)], rtol=0, atol=1e-10 * P)
        bw = np.zeros_like(bz)
        for s in range(pl.NC):
            c = pl.col(s, g)
            direct = c <= P // 2
            hc = c if direct else P - c
            for ky in range(P):
                kym = 0 if ky == 0 else P - ky
                z = bz[s * pl.CP + pl.spos(ky)]
                zm = np.conj(bz[pl.mirror(s, g) * pl.CP + pl.spos(kym)])
                row = ky if direct else kym
                ha, hb = Ha[row, hc], Hb[row, hc]
                if not direct:
                    ha, hb = np.conj(ha), np.conj(hb)
                bw[s * pl.CP + pl.spos(ky)] = (z + zm) / 2 * ha + (z - zm) / 2 * hb
        pl.inverse(bw)
        for s in range(pl.NC):
            for y in range(P):
                out[y, pl.col(s, g)] = bw[s * pl.CP + pl.pos(y)]
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-10 * np.abs(ref).max())
