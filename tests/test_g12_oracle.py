"""The oracle's geminal (G12) integrals and direct matrices, on the CPU.

The inter-particle potential of the reference's G12 path is libint2's
contracted Gaussian geminal V(r12) = sum_k c_k exp(-g_k r12^2)
(src/ints/Libint2Iface.cpp:2193-2540).  libint2 is not vendored, so the oracle's
integrals are pinned here by an independent computation: Cartesian Gaussians
and exp(-g (r1 - r2)^2) both factor over x, y, z, so a primitive integral is a
product of three two-dimensional Gaussian integrals of polynomials, which an
n-point Gauss-Hermite rule in each variable integrates exactly (degree <= 2n-1).
The direct matrices are pinned by the constant potential (g = 0), whose
integrals are products of overlaps: G = S tr(D S) + factor S D S.
"""
import numpy as np
import pytest

from openlowdin_gb300 import systems as S


def _carts(l):
    return [(l - i, i - j, j) for i in range(l + 1) for j in range(i + 1)]


def _one_dim(e, a4, x4, g, nodes, weights):
    """int int (x1-A)^ea (x1-B)^eb (x2-C)^ec (x2-D)^ed
       exp(-a (x1-A)^2 - b (x1-B)^2 - c (x2-C)^2 - d (x2-D)^2 - g (x1-x2)^2) dx1 dx2"""
    a, b, c, d = a4
    A, B, C, D = x4
    M = np.array([[a + b + g, -g], [-g, c + d + g]])
    rhs = np.array([a * A + b * B, c * C + d * D])
    z0 = np.linalg.solve(M, rhs)
    c0 = a * A * A + b * B * B + c * C * C + d * D * D - z0 @ M @ z0
    L = np.linalg.cholesky(M)
    Y1, Y2 = np.meshgrid(nodes, nodes, indexing="ij")
    Z = z0[:, None] + np.linalg.solve(L.T, np.stack([Y1.ravel(), Y2.ravel()]))
    x1, x2 = Z
    f = (x1 - A) ** e[0] * (x1 - B) ** e[1] * (x2 - C) ** e[2] * (x2 - D) ** e[3]
    return np.exp(-c0) / np.sqrt(np.linalg.det(M)) * np.sum(np.outer(weights, weights).ravel() * f)


def geminal_by_quadrature(l4, a4, origins, coefs, expos):
    nodes, weights = np.polynomial.hermite.hermgauss(12)
    out = []
    for ca in _carts(l4[0]):
        for cb in _carts(l4[1]):
            for cc in _carts(l4[2]):
                for cd in _carts(l4[3]):
                    v = 0.0
                    for ck, gk in zip(coefs, expos):
                        p = 1.0
                        for x in range(3):
                            p *= _one_dim((ca[x], cb[x], cc[x], cd[x]), a4, origins[:, x], gk, nodes, weights)
                        v += ck * p
                    out.append(v)
    return np.array(out)


CLASSES = [(0, 0, 0, 0), (1, 0, 0, 0), (1, 1, 0, 0), (1, 0, 1, 0), (2, 0, 0, 0), (1, 1, 1, 1),
           (2, 1, 1, 0), (2, 2, 1, 0), (2, 1, 2, 1), (2, 2, 2, 2)]


@pytest.mark.parametrize("l4", CLASSES)
def test_geminal_primitives_against_quadrature(oracle, l4):
    rng = np.random.default_rng(sum(l4) * 7 + l4[0])
    a4 = rng.uniform(0.3, 3.0, 4)
    origins = rng.normal(size=(4, 3))
    coefs, expos = [0.7, -0.3, 0.2, 1.1], [0.0, 0.4, 2.5, 9.0]
    ref = geminal_by_quadrature(l4, a4, origins, coefs, expos)
    got = oracle.g12_primitive(l4, a4, origins, coefs, expos)
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))


def _water_d():
    sysd = S.water(d_shell=True)
    return sysd["species"][0]


def test_constant_potential_intra_is_overlap_products(oracle):
    """V = c (g = 0): (ij|V|kl) = c S_ij S_kl, so G = c (S tr(DS) + factor S D S)."""
    sp = _water_d()
    b = oracle.Basis.from_shells(sp["shells"])
    Sm, _ = oracle.overlap_kinetic(b)
    rng = np.random.default_rng(3)
    X = rng.normal(size=Sm.shape) * 0.2
    D = X + X.T
    c, f = 0.37, -0.5
    G = oracle.g12_direct(b, D, f, [c], [0.0])
    ref = c * (Sm * np.sum(D * Sm) + f * Sm @ D @ Sm)
    assert np.max(np.abs(G - ref)) < 1e-10


def test_constant_potential_inter_is_overlap_products(oracle):
    sysd = S.water_cluster(1, seed=0, quantum_protons=True)
    ea, pa = sysd["species"][0], sysd["species"][1]
    be, bp = oracle.Basis.from_shells(ea["shells"]), oracle.Basis.from_shells(pa["shells"])
    Se, _ = oracle.overlap_kinetic(be)
    Sp, _ = oracle.overlap_kinetic(bp)
    rng = np.random.default_rng(4)
    X = rng.normal(size=Sp.shape) * 0.2
    Dp = X + X.T
    c = 0.8
    for sid, osid in ((1, 2), (2, 1)):   # both loop orders of the reference
        B = oracle.g12inter_direct(be, sid, bp, osid, Dp, [c], [0.0])
        ref = np.tril(c * Se * np.sum(Dp * Sp))
        # raw |v| < 1e-10 values are dropped (a few tiny overlap products)
        assert np.max(np.abs(B - ref)) < 1e-8
        assert np.all(np.triu(B, 1) == 0.0)


def test_direct_matrices_are_linear_in_the_potential(oracle):
    sp = _water_d()
    b = oracle.Basis.from_shells(sp["shells"])
    rng = np.random.default_rng(5)
    X = rng.normal(size=(b.nbf, b.nbf)) * 0.2
    D = X + X.T
    G1 = oracle.g12_direct(b, D, -1.0, [1.3], [0.6])
    G2 = oracle.g12_direct(b, D, -1.0, [-0.4], [3.0])
    G12 = oracle.g12_direct(b, D, -1.0, [1.3, -0.4], [0.6, 3.0])
    assert np.max(np.abs(G12 - (G1 + G2))) < 1e-12
