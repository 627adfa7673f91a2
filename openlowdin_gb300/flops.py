"""Frozen FLOP model of the integral kernels (used for roofline accounting).

For a shell-quartet class (la lb|lc ld) it counts the floating-point
operations the kernels of this library issue for one primitive quartet
(Obara-Saika vertical recursion on the bra, then on the ket, the Boys function
and the prefactors) plus, per contracted quartet, the horizontal transfers and
the digestion into the Fock-type outputs.  An FMA counts 2, add / mul 1, and a
transcendental (exp, sqrt, reciprocal) 1, so the count is a lower bound of the
pipe work.  The node enumeration replays eri.cuh exactly (same recursion axis
and the same m ranges), so a kernel that skips work cannot raise the count:
`achieved = sum_class quartets_evaluated(class) * F(class) / time`.
"""
from __future__ import annotations

from functools import lru_cache


def ncart(l):
    return (l + 1) * (l + 2) // 2


def coff(k):
    return k * (k + 1) * (k + 2) // 6


def _carts(total_max):
    out = []
    for k in range(total_max + 1):
        for i in range(k + 1):
            for j in range(i + 1):
                out.append((k - i, i - j, j))
    return out


def _dir(c):
    return 0 if c[0] > 0 else (1 if c[1] > 0 else 2)


@lru_cache(maxsize=None)
def vrr_flops(la, lb, lc, ld) -> int:
    L1, L2 = la + lb, lc + ld
    L = L1 + L2
    E = _carts(L1)
    F = _carts(L2)
    ops = 45                      # W, PA, WP, QC, WQ, |PQ|^2, rho, prefactor, reciprocals
    ops += 2 * 8 + 8 + 1          # Taylor Horner (FMA + mul per term) + table index
    ops += 2 + 3 * L              # exp and downward recursion
    ops += L + 1                  # [00|00]^(m) = pref * F_m
    for e in E[1:]:
        k = sum(e)
        ei = e[_dir(e)] - 1
        per = 3 + (5 if ei > 0 else 0)
        ops += per * (L - k + 1)
    for f in F[1:]:
        kf = sum(f)
        d = _dir(f)
        fi = f[d] - 1
        for e in E:
            ed = e[d]
            per = 3 + (5 if fi > 0 else 0) + (3 if ed > 0 else 0)
            ops += per * (L2 - kf + 1)
    nE = coff(L1 + 1) - coff(la)
    nF = coff(L2 + 1) - coff(lc)
    ops += nE * nF                # accumulation into X
    return ops


@lru_cache(maxsize=None)
def hrr_flops(la, lb, lc, ld) -> int:
    nF = coff(lc + ld + 1) - coff(lc)
    ops = 0
    for j in range(1, lb + 1):
        na = coff(la + lb - j + 1) - coff(la)
        ops += 2 * na * ncart(j) * nF
    nrow = ncart(la) * ncart(lb)
    for j in range(1, ld + 1):
        nc = coff(lc + ld - j + 1) - coff(lc)
        ops += 2 * nrow * nc * ncart(j)
    return ops


def digest_flops(la, lb, lc, ld, kind: str) -> int:
    n = ncart(la) * ncart(lb) * ncart(lc) * ncart(ld)
    if kind == "jk":          # six contractions of the quartet with density blocks
        return 6 * 2 * n
    if kind == "coupling":    # two contractions (both species)
        return 2 * 2 * n
    return 0


def quartet_flops(la, lb, lc, ld, kind="jk", nprim_quartets=1) -> int:
    return nprim_quartets * vrr_flops(la, lb, lc, ld) + hrr_flops(la, lb, lc, ld) + digest_flops(la, lb, lc, ld, kind)


PAIR_CLASSES = [(la, lb) for la in range(4) for lb in range(la + 1)]   # the library's ten pair classes


def class_table_flops(counts, kind="jk") -> float:
    """counts[cb][ck] quartets of (pair class cb | pair class ck) -> total FLOP."""
    tot = 0.0
    for cb, (la, lb) in enumerate(PAIR_CLASSES):
        for ck, (lc, ld) in enumerate(PAIR_CLASSES):
            c = counts[cb][ck]
            if c:
                tot += float(c) * quartet_flops(la, lb, lc, ld, kind)
    return tot
