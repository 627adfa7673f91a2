"""Seeded synthetic molecular systems for the benchmark workloads.

A system is plain data (a dict) so that the GPU library, the host SCF driver
and any checker can consume it alike:

    {"species": [{"name", "charge", "mass", "n_particles", "kappa", "eta",
                  "particles_fraction", "is_electron",
                  "shells": [(l, exponents, coefficients, origin_xyz), ...]}],
     "point_charges": [Z, ...], "point_positions": [[x, y, z], ...]}

Coordinates are bohr.  Shell order is insertion order (atoms in order, shells of
an atom in basis order), as the reference's Fortran constructor adds them
(src/ints/Libint2Interface.f90:382-448).  Species constants follow
lib/dataBases/constantsOfCoupling.lib: electrons kappa=-1, eta=2, fraction 1/2;
quantum protons (H_1) kappa=-1, eta=1, fraction 1.

Workloads (all basis sets uncontracted, even-tempered, Cartesian):
  water()        -- one water, O at the origin, O-H 1.809 bohr, HOH 104.5 deg;
                    O: s 0.15*2.6^k (k=0..7), p 0.2*2.8^k (k=0..3);
                    H: s 0.12*3^k (k=0..3), p 0.8.  34 functions, 10 electrons.
  water_cluster(n, seed, ...) -- n waters with uniform random rotations and
                    rejection-sampled translations (all O-O >= 5.1 bohr) in a
                    cube of edge 5.1*ceil(n^(1/3))*1.5 bohr.
                    quantum_protons=True: every H is a quantum proton (s 4, 8,
                    16, 24 and p 16 per proton, mass 1836.15267247), by default
                    each its own one-particle species; O stays a point charge.
                    4 waters -> e- 136 functions + 8 proton species of 7
                    functions (56 in total).
                    o_d=True: one Cartesian d shell (exponent 1.2) on O
                    (40 functions per water).
  chain_molecule(seed, ...) -- H/C/N/O self-avoiding chain, 3-30 atoms,
                    bonds U(2.0, 2.9) bohr, closed shell.
"""
from __future__ import annotations

import math

import numpy as np

PROTON_MASS = 1836.15267247
OH_BOHR = 1.809
HOH_DEG = 104.5

O_S = [0.15 * 2.6 ** k for k in range(8)]
O_P = [0.2 * 2.8 ** k for k in range(4)]
H_S = [0.12 * 3.0 ** k for k in range(4)]
H_P = [0.8]
O_D = [1.2]
PROTON_S = [4.0, 8.0, 16.0, 24.0]
PROTON_P = [16.0]

Z_OF = {"H": 1, "C": 6, "N": 7, "O": 8}


def _heavy_shells(pos, d_shell=False):
    sh = [(0, [a], [1.0], list(pos)) for a in O_S]
    sh += [(1, [a], [1.0], list(pos)) for a in O_P]
    if d_shell:
        sh += [(2, [a], [1.0], list(pos)) for a in O_D]
    return sh


def _h_shells(pos):
    return [(0, [a], [1.0], list(pos)) for a in H_S] + [(1, [a], [1.0], list(pos)) for a in H_P]


def _proton_shells(pos):
    return [(0, [a], [1.0], list(pos)) for a in PROTON_S] + [(1, [a], [1.0], list(pos)) for a in PROTON_P]


def electron_species(shells, n_electrons):
    return {"name": "E-", "charge": -1.0, "mass": 1.0, "n_particles": int(n_electrons),
            "kappa": -1.0, "eta": 2.0, "particles_fraction": 0.5, "is_electron": True,
            "shells": shells}


def uhf_electron_species(shells, n_electrons, multiplicity=1):
    """Open-shell (UHF) electrons as the reference runs them: two species,
    E-ALPHA and E-BETA, over the same shells, each with kappa = -1, eta = 1
    (one particle per orbital, exchange factor -1), coupled to each other by
    the inter-species Coulomb matrix like any other species pair
    (src/core/Species.f90, constantsOfCoupling.lib).  n_alpha - n_beta =
    multiplicity - 1."""
    n_beta = (int(n_electrons) - (int(multiplicity) - 1)) // 2
    n_alpha = int(n_electrons) - n_beta
    if n_beta < 0 or n_alpha - n_beta != int(multiplicity) - 1:
        raise ValueError(f"{n_electrons} electrons cannot have multiplicity {multiplicity}")
    out = []
    for name, n in (("E-ALPHA", n_alpha), ("E-BETA", n_beta)):
        sp = electron_species(shells, n)
        sp.update(name=name, eta=1.0, particles_fraction=1.0)
        out.append(sp)
    return out


def proton_species(shells, n_protons, name="H_1"):
    return {"name": name, "charge": 1.0, "mass": PROTON_MASS, "n_particles": int(n_protons),
            "kappa": -1.0, "eta": 1.0, "particles_fraction": 1.0, "is_electron": False,
            "shells": shells}


def water_geometry():
    """O at the origin, H atoms in the xz plane."""
    h = math.radians(HOH_DEG) / 2.0
    O = np.zeros(3)
    H1 = np.array([OH_BOHR * math.sin(h), 0.0, OH_BOHR * math.cos(h)])
    H2 = np.array([-OH_BOHR * math.sin(h), 0.0, OH_BOHR * math.cos(h)])
    return O, H1, H2


def _random_rotation(rng):
    """Uniform random rotation from a uniform unit quaternion."""
    u1, u2, u3 = rng.random(3)
    q = np.array([math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                  math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3)])
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def cluster_positions(n_waters: int, seed: int, min_oo: float = 5.1):
    """List of (O, H1, H2) positions, seeded (numpy PCG64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    edge = min_oo * math.ceil(n_waters ** (1.0 / 3.0) - 1e-9) * 1.5
    O0, H10, H20 = water_geometry()
    mols = []
    for _ in range(n_waters):
        for _attempt in range(100000):
            t = rng.random(3) * edge
            if all(np.linalg.norm(t - m[0]) >= min_oo for m in mols):
                break
        else:
            raise RuntimeError("could not place water")
        R = _random_rotation(rng)
        mols.append((t + R @ O0, t + R @ H10, t + R @ H20))
    return mols


def water(d_shell=False):
    return water_cluster(1, seed=0, quantum_protons=False, o_d=d_shell, place=False)


def water_cluster(n_waters: int, seed: int = 0, quantum_protons=False, o_d=False, place=True,
                  proton_species_mode="per_proton"):
    """proton_species_mode: "per_proton" gives every quantum proton its own
    one-particle species (H-1_1, H-2_1, ..., the convention of the reference's
    APMO tests, e.g. H-a_1 / H-b_1 in test/H2O.APMO.MP2.lowdin); "single" puts
    all protons in one H_1 species (fermions with exchange)."""
    mols = cluster_positions(n_waters, seed) if place else [water_geometry()]
    e_shells, p_shells, Z, R = [], [], [], []
    for O, H1, H2 in mols:
        e_shells += _heavy_shells(O, o_d)
        e_shells += _h_shells(H1) + _h_shells(H2)
        Z.append(8.0); R.append(list(O))
        if quantum_protons:
            p_shells.append(_proton_shells(H1))
            p_shells.append(_proton_shells(H2))
        else:
            Z += [1.0, 1.0]; R += [list(H1), list(H2)]
    species = [electron_species(e_shells, 10 * len(mols))]
    if quantum_protons:
        if proton_species_mode == "single":
            species.append(proton_species([s for p in p_shells for s in p], 2 * len(mols)))
        else:
            species += [proton_species(p, 1, name=f"H-{k + 1}_1") for k, p in enumerate(p_shells)]
    return {"species": species, "point_charges": Z, "point_positions": R,
            "name": f"water{len(mols)}" + ("-apmo" if quantum_protons else "") + ("-d" if o_d else "")}


def chain_molecule(seed: int, n_atoms=None, min_atoms=3, max_atoms=30):
    """H/C/N/O self-avoiding chain (p = .5/.25/.125/.125), bonds U(2.0, 2.9)
    bohr, every atom >= 2.0 bohr from all others; one terminal H added or
    removed to make the electron count even.  C/N/O carry the O pattern, H the
    H pattern."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = int(n_atoms) if n_atoms is not None else int(rng.integers(min_atoms, max_atoms + 1))
    elems = rng.choice(["H", "C", "N", "O"], size=n, p=[0.5, 0.25, 0.125, 0.125]).tolist()
    pos = [np.zeros(3)]
    while len(pos) < n:
        for _attempt in range(1000):
            v = rng.normal(size=3)
            v /= np.linalg.norm(v)
            cand = pos[-1] + v * rng.uniform(2.0, 2.9)
            if all(np.linalg.norm(cand - p) >= 2.0 for p in pos):
                pos.append(cand)
                break
        else:
            pos = pos[:-1] if len(pos) > 1 else pos
    nel = sum(Z_OF[e] for e in elems)
    if nel % 2:
        if elems[-1] == "H" and len(elems) > 3:
            elems.pop(); pos.pop()
        else:
            for _attempt in range(1000):
                v = rng.normal(size=3)
                v /= np.linalg.norm(v)
                cand = pos[-1] + v * rng.uniform(2.0, 2.9)
                if all(np.linalg.norm(cand - p) >= 2.0 for p in pos):
                    pos.append(cand); elems.append("H")
                    break
    shells, Z, R = [], [], []
    for e, p in zip(elems, pos):
        shells += _h_shells(p) if e == "H" else _heavy_shells(p)
        Z.append(float(Z_OF[e])); R.append(list(p))
    nel = int(sum(Z))
    return {"species": [electron_species(shells, nel)], "point_charges": Z, "point_positions": R,
            "name": f"chain{len(elems)}-s{seed}"}


def chain_for_basis(seed: int, target_nbf: int, max_atoms: int = 400):
    """The chain generator grown (same seed, more atoms) until the electron
    basis reaches target_nbf functions."""
    for n in range(3, max_atoms + 1):
        m = chain_molecule(seed, n_atoms=n)
        if nbasis(m["species"][0]) >= target_nbf:
            return m
    return m


def n_core(sysd) -> int:
    """Frozen-core orbitals: one 1s orbital per atom heavier than He."""
    return int(sum(1 for z in sysd["point_charges"] if z > 2.0))


def nbasis(species) -> int:
    return int(sum((l + 1) * (l + 2) // 2 for l, _, _, _ in species["shells"]))
