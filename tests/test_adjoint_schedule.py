"""The unit schedule of the ordered module-shared adjoint, restated on the
CPU (no GPU): ``OrdSchedule`` in ``j-ubik_gb300/csrc/fused.cu`` and the spill
lookup of its per-patch kernel.  Every unit is taken exactly once; every
patch has exactly one CTA that holds its module 0 and writes its accumulator;
and the lookup names exactly the CTAs whose tail range continues the patch,
in CTA order (the order the partial sums are added in)."""
import itertools

import pytest


def schedule(G, M, patches):
    rounds = patches // G
    tail0 = rounds * G * M
    tu = (patches - rounds * G) * M
    Gt = min(G, tu)

    def tlo(b):
        return tail0 + tu if b >= Gt else tail0 + b * tu // Gt

    return rounds, tail0, tu, Gt, tlo


@pytest.mark.parametrize("G, M, patches", [
    c for c in itertools.product([1, 3, 7, 152, 304], [2, 3, 7], [1, 4, 9, 64, 768, 1000])
    if c[0] <= c[1] * c[2]])
def test_ordered_adjoint_schedule(G, M, patches):
    rounds, tail0, tu, Gt, tlo = schedule(G, M, patches)
    seen, owners, spills = set(), {}, {}
    for b in range(G):
        cnt = rounds * M + tlo(b + 1) - tlo(b)
        for t in range(cnt):
            g = (b + (t // M) * G) * M + t % M if t < rounds * M else tlo(b) + t - rounds * M
            assert g not in seen
            seen.add(g)
            m, tail = g % M, t >= rounds * M
            last = m == M - 1 or t == cnt - 1
            owner = (not tail) or g - m >= tlo(b)
            if last:
                if owner:
                    owners[g // M] = owners.get(g // M, 0) + 1
                else:
                    spills.setdefault(g // M, []).append(b)
    assert seen == set(range(patches * M))
    assert all(owners.get(p) == 1 for p in range(patches))
    for p in range(patches):  # the per-patch kernel's lookup
        u0, b, n = p * M, 0, 0
        if u0 >= tail0 and tu > 0:
            b = ((u0 + 1 - tail0) * Gt + tu - 1) // tu
            while b + n < Gt and tlo(b + n) < u0 + M:
                n += 1
        assert list(range(b, b + n)) == spills.get(p, [])
