"""Systems of the reference's golden tests, built from tests/golden/golden.json."""
import numpy as np

from openlowdin_gb300 import systems as S


def _shells(golden, key, pos):
    return [(s["l"], s["exponents"], s["coefficients"], list(pos)) for s in golden["basis"][key]]


def h2o_boa(golden):
    """test/H2O.BOA.DIRECT: RHF, 6-311G electrons, classical O and H."""
    geo = golden["geometry"]["H2O.BOA.DIRECT"]
    shells, Z, R = [], [], []
    for r in geo:
        if r["particle"] == "e-[O]":
            shells += _shells(golden, "6-311G:O", r["position_bohr"])
        elif r["particle"] == "e-[H]":
            shells += _shells(golden, "6-311G:H", r["position_bohr"])
        elif r["basis"] == "dirac":
            Z.append({"O": 8.0, "H_1": 1.0}[r["particle"]]); R.append(r["position_bohr"])
    return {"species": [S.electron_species(shells, 10)], "point_charges": Z, "point_positions": R,
            "name": "H2O.BOA"}


def h2o_apmo(golden):
    """test/H2O.APMO.MP2: 6-311G electrons, classical O, two quantum protons
    H-a_1 / H-b_1 (one particle each) with NAKAI-5-SPD."""
    geo = golden["geometry"]["H2O.APMO.MP2"]
    shells, Z, R, prot = [], [], [], []
    for r in geo:
        if r["particle"] == "e-[O]":
            shells += _shells(golden, "6-311G:O", r["position_bohr"])
        elif r["particle"] == "e-[H]":
            shells += _shells(golden, "6-311G:H", r["position_bohr"])
        elif r["basis"] == "dirac":
            Z.append(8.0); R.append(r["position_bohr"])
        else:
            prot.append(S.proton_species(_shells(golden, "NAKAI-5-SPD:H_1", r["position_bohr"]), 1,
                                         name=r["particle"].upper()))
    return {"species": [S.electron_species(shells, 10)] + prot, "point_charges": Z, "point_positions": R,
            "name": "H2O.APMO"}


_Z = {"H": 1.0, "H_1": 1.0, "C": 6.0, "N": 7.0, "O": 8.0, "Ne": 10.0}


def uhf_system(golden, test, electron_basis, proton_basis):
    """An open-shell APMO input of the reference as a UHF system: electrons of
    every e-(X) centre in `electron_basis`, classical point charges for the
    'dirac' rows, one quantum proton species per H_1 row.  Electron count
    sum Z + addParticles; multiplicity M gives n_alpha - n_beta = M - 1."""
    geo = golden["geometry"][test]
    shells, Z, R, prot = [], [], [], []
    n_el, add, mult = 0, 0, 1
    for r in geo:
        part = r["particle"]
        if part.startswith("e-"):
            el = part[3:-1]
            shells += _shells(golden, f"{electron_basis}:{el}", r["position_bohr"])
            n_el += int(_Z[el])
            add += r.get("add_particles", 0)
            mult = max(mult, r.get("multiplicity", 1))
        elif r["basis"] == "dirac":
            Z.append(_Z[part]); R.append(r["position_bohr"])
        else:
            prot.append(S.proton_species(_shells(golden, f"{proton_basis}:H_1", r["position_bohr"]), 1,
                                         name=part.upper()))
    return {"species": S.uhf_electron_species(shells, n_el + add, mult) + prot, "point_charges": Z,
            "point_positions": R, "name": test}


def h2o_apmo_uhf(golden):
    """test/H2O.APMO.UHF.DIRECT: the H2O.APMO system with UHF electrons."""
    sysd = h2o_apmo(golden)
    e = sysd["species"][0]
    sysd["species"] = S.uhf_electron_species(e["shells"], 10, 1) + sysd["species"][1:]
    return sysd


def hf_apmo(golden):
    """test/HF.APMO: HF with cc-pVTZ electrons (an f shell on F), classical F,
    one quantum proton H_1 (DZSPDN)."""
    geo = golden["geometry"]["HF.APMO"]
    shells, Z, R, prot = [], [], [], []
    for r in geo:
        part = r["particle"]
        if part.startswith("e-"):
            shells += _shells(golden, "CC-PVTZ:" + part[3:-1], r["position_bohr"])
        elif r["basis"] == "dirac":
            Z.append(9.0); R.append(r["position_bohr"])
        else:
            prot.append(S.proton_species(_shells(golden, "DZSPDN:H_1", r["position_bohr"]), 1, name=part.upper()))
    return {"species": [S.electron_species(shells, 10)] + prot, "point_charges": Z, "point_positions": R,
            "name": "HF.APMO"}


def g12_system(golden, test):
    """A TIP4P-style input of the reference (test/TIP4P-dimer-*-direct): one
    quantum species per particle name with a basis (UHF: kappa = -1, eta = 1,
    one particle per orbital), the 'dirac' rows as point charges, the
    EXTERPOTENTIAL entries as external potentials and the INTERPOTENTIAL
    entries as G12 pair potentials."""
    inp = golden["g12_inputs"][test]
    assert inp["method"] == "UHF"
    names, rows, Z, R = [], {}, [], []
    for r in inp["particles"]:
        if r["basis"] == "dirac":
            Z.append(r["charge"]); R.append(r["position_bohr"])
            continue
        if r["particle"] not in rows:
            names.append(r["particle"]); rows[r["particle"]] = []
        rows[r["particle"]].append(r)
    species = []
    for nm in names:
        shells = []
        for r in rows[nm]:
            shells += [(s["l"], s["exponents"], s["coefficients"], list(r["position_bohr"])) for s in inp["basis"][nm]]
        r0 = rows[nm][0]
        species.append({"name": nm, "charge": r0["charge"], "mass": r0["mass"], "n_particles": len(rows[nm]),
                        "kappa": -1.0, "eta": 1.0, "particles_fraction": 1.0, "is_electron": False,
                        "shells": shells})

    def comps(pot, key):
        c = inp["potentials"][pot][key]
        assert all(x["l"] == 0 for x in c)
        return [x["coefficient"] for x in c], [x["exponent"] for x in c], [x["origin"] for x in c]

    ext = []
    for e in inp["external"]:
        c, g, o = comps(e["potential"], e["species"])
        ext.append({"species": names.index(e["species"]), "coefficients": c, "exponents": g, "origins": o})
    inter = []
    for e in inp["inter"]:
        a, b = e["species"]
        key = a + b if a + b in inp["potentials"][e["potential"]] else b + a
        c, g, _ = comps(e["potential"], key)
        inter.append({"species": [names.index(a), names.index(b)], "coefficients": c, "exponents": g})
    return {"species": species, "point_charges": Z, "point_positions": R, "external_potentials": ext,
            "interpotentials": inter, "name": test}


def g12_components(P, names, sysd, Vext, Vfix, Ginter, Gintra_coulomb, Gintra):
    """The energy components the TIP4P checkers read, from converged densities:
    'X Ext Pot' tr P V_ext, 'X/Fixed interact.' tr P q V_fixed, 'X/Y Hartree'
    tr P_X J_XY, and for a species with two particles 'X/X Hartree'
    tr P J[P] / 2 and 'X Exchange' tr P (G - J[P]) / 2."""
    out = {}
    for i, nm in enumerate(names):
        out[f"{nm} Ext Pot"] = float(np.sum(P[i] * Vext[i]))
        out[f"{nm}/Fixed interact."] = float(np.sum(P[i] * Vfix[i]))
        if Gintra[i] is not None:
            out[f"{nm}/{nm} Hartree"] = 0.5 * float(np.sum(P[i] * Gintra_coulomb[i]))
            out[f"{nm} Exchange"] = 0.5 * float(np.sum(P[i] * (Gintra[i] - Gintra_coulomb[i])))
    for (i, j), B in Ginter.items():
        out[f"{names[i]}/{names[j]} Hartree"] = float(np.sum(P[i] * B))
    return out


def h2o_apmo_two_protons(golden):
    """test/H2O.APMO.iter0-iter3: 6-31G electrons, classical O, both protons in
    one species H_1 (two particles, NAKAI-3-SP, kappa = -1, eta = 1)."""
    geo = golden["geometry"]["H2O.APMO.iter0"]
    shells, Z, R, pshells = [], [], [], []
    for r in geo:
        part = r["particle"]
        if part.startswith("e-"):
            shells += _shells(golden, "6-31G:" + part[3:-1], r["position_bohr"])
        elif r["basis"] == "dirac":
            Z.append(_Z[part]); R.append(r["position_bohr"])
        else:
            pshells += _shells(golden, "NAKAI-3-SP:H_1", r["position_bohr"])
    return {"species": [S.electron_species(shells, 10), S.proton_species(pshells, 2)], "point_charges": Z,
            "point_positions": R, "name": "H2O.APMO.iter"}


def psh(golden):
    """test/PsH.P3: the two electrons of H^- (e-(H) with addParticles=1, UHF,
    cc-pVTZ), the H nucleus as a point charge and one positron species
    (charge +1, mass 1, kappa = -1, eta = 1; e+-H-7SP-aug-cc-pVTZ)."""
    geo = golden["geometry"]["PsH.P3"]
    e, nuc, pos = geo
    electrons = S.uhf_electron_species(_shells(golden, "CC-PVTZ:H", e["position_bohr"]), 1 + e["add_particles"], 1)
    positron = {"name": "E+", "charge": 1.0, "mass": 1.0, "n_particles": 1, "kappa": -1.0, "eta": 1.0,
                "particles_fraction": 1.0, "is_electron": False,
                "shells": _shells(golden, "E+-H-7SP-AUG-CC-PVTZ:E+", pos["position_bohr"])}
    return {"species": electrons + [positron], "point_charges": [_Z[nuc["particle"]]],
            "point_positions": [nuc["position_bohr"]], "name": "PsH.P3"}


def he_potentials(golden):
    """test/He.POTENTIALS: the two electrons of He (e-(He), 6-31G, UHF) with no
    nucleus; the fitted potential HEE acts on each electron species
    (EXTERPOTENTIAL) and the fitted EE replaces their Coulomb interaction
    (INTERPOTENTIAL: G12 pair potentials)."""
    r = golden["geometry"]["He.POTENTIALS"][0]
    species = S.uhf_electron_species(_shells(golden, "6-31G:He", r["position_bohr"]), 2, 1)
    names = [s["name"] for s in species]
    inp = golden["g12_inputs"]["He.POTENTIALS"]
    assert inp["method"] == "UHF"
    pots = inp["potentials"]

    def comps(pot, key):
        c = pots[pot.upper()][key]
        assert all(x["l"] == 0 for x in c)
        return [x["coefficient"] for x in c], [x["exponent"] for x in c], [x["origin"] for x in c]

    ext = []
    for e in inp["external"]:
        c, g, o = comps(e["potential"], e["species"])
        ext.append({"species": names.index(e["species"]), "coefficients": c, "exponents": g, "origins": o})
    inter = []
    for e in inp["inter"]:
        a, b = e["species"]
        c, g, _ = comps(e["potential"], a + b)
        inter.append({"species": [names.index(a), names.index(b)], "coefficients": c, "exponents": g})
    return {"species": species, "point_charges": [], "point_positions": [], "external_potentials": ext,
            "interpotentials": inter, "name": "He.POTENTIALS"}


def nh3_apmo_three_protons(golden):
    """test/NH3.APMO.convBoth: 6-31G* electrons, classical N, the three protons
    in one species H_1 (three particles, DZSPNB)."""
    geo = golden["geometry"]["NH3.APMO.convBoth"]
    shells, Z, R, pshells = [], [], [], []
    for r in geo:
        part = r["particle"]
        if part.startswith("e-"):
            shells += _shells(golden, "6-31G.D:" + part[3:-1], r["position_bohr"])
        elif r["basis"] == "dirac":
            Z.append(_Z[part]); R.append(r["position_bohr"])
        else:
            pshells += _shells(golden, "DZSPNB:H_1", r["position_bohr"])
    return {"species": [S.electron_species(shells, 10), S.proton_species(pshells, 3)], "point_charges": Z,
            "point_positions": R, "name": "NH3.APMO.convBoth"}


def c60_system(golden, test):
    """test/He2-C60potential-NOCI / He3-: one species per particle name (HEA3,
    HEB3; one s function per particle) with the particle database's charge and
    coupling constants and the input's mass, the C60 cage as the external
    potential of every species (expanded from terms x centres), the fitted
    He-He potential as the G12 pair potentials, and the point particle N0."""
    inp = golden["g12_inputs"][test]
    assert inp["method"] == "UHF"
    names, rows, Z, R = [], {}, [], []
    for r in inp["particles"]:
        if r["basis"] == "dirac":
            Z.append(r["charge"]); R.append(r["position_bohr"])
            continue
        if r["particle"] not in rows:
            names.append(r["particle"]); rows[r["particle"]] = []
        rows[r["particle"]].append(r)
    species = []
    for nm in names:
        shells = [(s["l"], s["exponents"], s["coefficients"], list(r["position_bohr"]))
                  for r in rows[nm] for s in inp["basis"][nm]]
        r0 = rows[nm][0]
        species.append(dict(inp["constants"][nm], name=nm, charge=r0["charge"], mass=r0["mass"],
                            n_particles=len(rows[nm]), is_electron=False, shells=shells))
    ext = []
    for e in inp["external"]:
        f = inp["potentials"][e["potential"]][e["species"]]
        terms = [(g, c, o) for g, c in f["terms"] for o in f["centers"]]
        ext.append({"species": names.index(e["species"]), "coefficients": [t[1] for t in terms],
                    "exponents": [t[0] for t in terms], "origins": [t[2] for t in terms]})
    inter = []
    for e in inp["inter"]:
        a, b = e["species"]
        c = inp["potentials"][e["potential"]][a + b]
        assert all(x["l"] == 0 for x in c)
        inter.append({"species": [names.index(a), names.index(b)], "coefficients": [x["coefficient"] for x in c],
                      "exponents": [x["exponent"] for x in c]})
    return {"species": species, "point_charges": Z, "point_positions": R, "external_potentials": ext,
            "interpotentials": inter, "name": test}
