"""Systems of the reference's golden tests, built from tests/golden/golden.json."""
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


_Z = {"H": 1.0, "O": 8.0}


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
