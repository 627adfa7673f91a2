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
