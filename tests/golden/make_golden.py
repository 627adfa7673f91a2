"""Generate tests/golden/golden.json from an openLOWDIN source tree.

Run once in a container that has the reference tree:

    python tests/golden/make_golden.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to $LOWDIN_REFERENCE, else /root/reference.

It extracts, as data:
  * the basis-set entries the golden tests use from ``lib/basis`` (6-311G for
    H and O electrons, NAKAI-5-SPD for quantum protons),
  * the geometries of the golden inputs ``test/H2O.BOA.DIRECT.lowdin``,
    ``test/H2O.APMO.MP2.lowdin`` (Angstrom, converted with AMSTRONG =
    0.52917724924 bohr from ``src/core/Units.f90:37``),
  * the golden values asserted by the checkers ``test/H2O.BOA.DIRECT.py``,
    ``test/H2O.BOA.MP2.DIRECT.py``, ``test/H2O.APMO.MP2.py``,
    ``test/H2O.APMO.UHF.DIRECT.py``, ``test/H2O.APMO.UMP2.DIRECT.py`` (the
    last two use the geometry of ``test/H2O.APMO.MP2.lowdin``),
  * for open-shell UHF: the inputs and checkers ``test/HOO+.ROCI-HF`` (triplet
    HOO+, cc-pVDZ electrons, DZSPNB proton), ``test/H3+.FCI`` (6-31G** electrons,
    DZSPDN proton) and ``test/H.APMO.READCOEFF`` (one electron, cc-pVDZ, DZSNB
    proton) with their bases (only the SCF energy of these checkers is used),
  * ``test/HF.APMO`` (HF with cc-pVTZ electrons, f shell on F, and a DZSPDN
    quantum proton): geometry, bases and the checker's HF and MP2 energies,
  * ``test/H2O.APMO.iter0``-``iter3`` (6-31G electrons, one species of two
    NAKAI-3-SP protons), ``test/NH3.APMO.convBoth`` (6-31G* electrons, one
    species of three DZSPNB protons; the values of its siblings convDens and
    convEne too), ``test/PsH.P3`` (UHF electrons of H^- with cc-pVTZ, a
    positron species) and ``test/He.POTENTIALS`` (UHF He electrons whose
    nucleus is the fitted external potential HEE and whose electron-electron
    interaction is the G12 potential EE, both from ``lib/potentials``):
    geometries, bases, potentials and the checkers' HF energies,
  * ``test/He2-C60potential-NOCI`` and ``He3-`` (helium atoms as quantum
    particles in a C60 cage fitted as 25 Gaussian terms at each of the 60
    carbon centres, lib/potentials HE2C60-IH-1P / -2P): geometry, basis,
    potentials (stored as terms x centres, checked exact), particle constants
    and the checkers' HF energies (their NOCI values are not used),
  * the HF energies of ``test/H2O.APMO.UP2``, ``test/H2O.APMO.FCI``,
    ``test/CO.CISD-dipole``, ``test/Ne.CISD``, ``test/H2O.BOA`` and
    ``test/H2O.BOA.UMP2`` (their post-HF values are not used),
  * the UHF inputs ``test/H2.APMO.UEN`` (cc-pVTZ electrons, NAKAI-3-SPD
    protons) and ``test/H2O.BOA.UEN`` (6-311++G** electrons): geometry, bases
    and the checkers' HF and MP2 energies (their Epstein-Nesbet values are
    not used),
  * the G12 tests ``test/TIP4P-dimer-{singlet,triplet}-direct`` (two quantum
    protons of a TIP4P water dimer under fitted Gaussian potentials): the
    geometry (bohr, ``units="BOHRS"``) with charges and masses, the charge of
    the point particle N0 from ``lib/dataBases/elementalParticles.lib``, the
    input's own BASIS block, its POTENTIAL blocks, the EXTERPOTENTIAL /
    INTERPOTENTIAL assignments and the checkers' values.
The GPU machine has no reference tree, so the tests read only the JSON written here.
"""
import json
import os
import re
import sys

ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LOWDIN_REFERENCE", "/root/reference")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
BOHR = 0.52917724924  # src/core/Units.f90:37


def read_basis(fname, element, symbol):
    """Parse one entry 'O-<ELEMENT> <SYMBOL> (<NAME>) BASIS TYPE: n' of a lowdin
    basis file: '#' line, shell count, then per shell 'id l nprim' and nprim
    'exponent coefficient' rows (src/core/BasisSet.f90:180-250)."""
    lines = open(os.path.join(ROOT, "lib", "basis", fname)).read().splitlines()
    head = re.compile(r"^O-%s\s+%s\s+\(" % (re.escape(element), re.escape(symbol)))
    for i, ln in enumerate(lines):
        if head.match(ln.strip()):
            j = i + 1
            while lines[j].strip().startswith("#"):
                j += 1
            nsh = int(lines[j].split()[0]); j += 1
            shells = []
            for _ in range(nsh):
                _, l, npr = (int(x) for x in lines[j].split()[:3]); j += 1
                ex, co = [], []
                for _ in range(npr):
                    a, c = lines[j].split()[:2]; j += 1
                    ex.append(float(a.replace("D", "E"))); co.append(float(c.replace("D", "E")))
                shells.append({"l": l, "exponents": ex, "coefficients": co})
            return shells
    raise KeyError(f"{element} {symbol} not in {fname}")


def read_geometry(name):
    rows = []
    txt = open(os.path.join(ROOT, "test", name)).read()
    block = txt.split("GEOMETRY")[1]
    for ln in block.splitlines()[1:]:
        ln = ln.strip()
        if not ln or ln.startswith("END"):
            break
        parts = ln.split()
        rec = {"particle": parts[0], "basis": parts[1],
               "position_bohr": [float(x) / BOHR for x in parts[2:5]]}
        m = re.search(r"(?<![A-Za-z])m\s*=\s*([0-9.Ee+-]+)", ln)
        if m:
            rec["mass"] = float(m.group(1))
        for key, name in (("addParticles", "add_particles"), ("multiplicity", "multiplicity")):
            m = re.search(key + r"\s*=\s*([-0-9]+)", ln, re.IGNORECASE)
            if m:
                rec[name] = int(m.group(1))
        rows.append(rec)
    return rows


def particle_charge(symbol):
    """CHARGE of a &PARTICLE entry of lib/dataBases/elementalParticles.lib."""
    txt = open(os.path.join(ROOT, "lib", "dataBases", "elementalParticles.lib")).read()
    for blk in txt.split("&PARTICLE")[1:]:
        m = re.search(r'SYMBOL\s*=\s*"([^"]+)"', blk)
        if m and m.group(1) == symbol:
            return float(re.search(r"CHARGE\s*=\s*([-0-9.Ee+]+)", blk).group(1))
    raise KeyError(symbol)


def coupling_constants(symbol):
    """KAPPA, ETA and PARTICLESFRACTION of a &SPECIE entry of
    lib/dataBases/constantsOfCoupling.lib."""
    txt = open(os.path.join(ROOT, "lib", "dataBases", "constantsOfCoupling.lib")).read()
    for blk in txt.split("&SPECIE")[1:]:
        m = re.search(r'SYMBOL\s*=\s*"([^"]+)"', blk)
        if m and m.group(1) == symbol:
            get = lambda k: float(re.search(k + r"\s*=\s*([-0-9.Ee+]+)", blk).group(1))
            return {"kappa": get("KAPPA"), "eta": get("ETA"), "particles_fraction": get("PARTICLESFRACTION")}
    raise KeyError(symbol)


def factored(comps):
    """A potential whose components are every (exponent, coefficient) term at
    every centre, term-major as in the file, stored as the two lists; the
    expansion is checked to give the file's components exactly."""
    terms, centers = [], []
    for c in comps:
        assert c["l"] == 0
        if [c["exponent"], c["coefficient"]] not in terms:
            terms.append([c["exponent"], c["coefficient"]])
        if c["origin"] not in centers:
            centers.append(c["origin"])
    assert [{"l": 0, "exponent": g, "coefficient": k, "origin": o} for g, k in terms for o in centers] == comps
    return {"terms": terms, "centers": centers}


def read_c60_input(name):
    """test/He{2,3}-C60potential-NOCI: helium atoms as quantum particles
    (HEA3 / HEB3, one s function each from lib/basis/HE2-1S) inside a C60
    cage given as the external potential HE2C60-IH-1P (25 terms at each of
    the 60 carbon centres) and interacting through HE2C60-IH-2P; charges and
    masses of lib/dataBases, the input's m= overriding the mass."""
    txt = open(os.path.join(ROOT, "test", name + ".lowdin")).read()
    assert re.search(r'units\s*=\s*"BOHRS"', txt)
    particles, names = [], []
    for ln in read_block(txt, "GEOMETRY", "END GEOMETRY").strip().splitlines():
        t = ln.split()
        rec = {"particle": t[0], "basis": t[1], "position_bohr": [float(x) for x in t[2:5]],
               "charge": particle_charge(t[0])}
        m = re.search(r"(?<![A-Za-z])m\s*=\s*([0-9.Ee+-]+)", ln)
        if m:
            rec["mass"] = float(m.group(1))
        if t[1] != "dirac" and t[0] not in names:
            names.append(t[0])
        particles.append(rec)
    asg = read_assignments(txt)
    ext = {e["potential"] for e in asg["external"]}
    inter = {e["potential"] for e in asg["inter"]}
    pots = {p: {k: factored(v) for k, v in read_potential_file(p.upper(), tuple(names)).items()} for p in ext}
    pots.update({p: read_potential_file(p.upper(), tuple(a + b for a in names for b in names)) for p in inter})
    basis = {n: read_basis(next(r["basis"] for r in particles if r["particle"] == n), "HELIUM", n) for n in names}
    return dict(asg, particles=particles, basis=basis, potentials=pots,
                constants={n: coupling_constants(n) for n in names})


def read_block(txt, head, tail):
    return txt.split(head, 1)[1].split(tail, 1)[0]


def read_g12_input(name):
    """One TIP4P-style input: particles, inline basis, Gaussian potentials.

    A POTENTIAL block holds, per 'O-<key>' entry, a component count, then per
    component an 'id l' line, an 'exponent coefficient' line and an origin line
    (the reader is src/core/GTFPotential.f90:155-307; it sets every
    component to l = 0 and interpotential origins to zero)."""
    txt = open(os.path.join(ROOT, "test", name + ".lowdin")).read()
    units = re.search(r'units\s*=\s*"([A-Za-z]+)"', txt)
    scale = 1.0 if units and units.group(1).upper().startswith("BOHR") else 1.0 / BOHR
    particles = []
    for ln in read_block(txt, "GEOMETRY", "END GEOMETRY").strip().splitlines():
        t = ln.split()
        if len(t) < 5:
            continue
        rec = {"particle": t[0], "basis": t[1], "position_bohr": [float(x) * scale for x in t[2:5]]}
        m = re.search(r"(?<![A-Za-z])q\s*=\s*([-0-9.Ee+]+)", ln)
        rec["charge"] = float(m.group(1)) if m else particle_charge(t[0])
        m = re.search(r"(?<![A-Za-z])m\s*=\s*([0-9.Ee+-]+)", ln)
        if m:
            rec["mass"] = float(m.group(1))
        particles.append(rec)
    basis = {}
    lines = read_block(txt, "\nBASIS ", "END BASIS").splitlines()
    for i, ln in enumerate(lines):
        m = re.match(r"^O-\S+\s+(\S+)\s+\(", ln.strip())
        if not m:
            continue
        j = i + 1
        nsh = int(lines[j].split()[0]); j += 1
        shells = []
        for _ in range(nsh):
            _, l, npr = (int(x) for x in lines[j].split()[:3]); j += 1
            ex, co = [], []
            for _ in range(npr):
                a, c = lines[j].split()[:2]; j += 1
                ex.append(float(a)); co.append(float(c))
            shells.append({"l": l, "exponents": ex, "coefficients": co})
        basis[m.group(1)] = shells
    potentials = {}
    for blk in txt.split("\nPOTENTIAL ")[1:]:
        lines = blk.split("END POTENTIAL")[0].splitlines()
        potentials[lines[0].strip()] = potential_entries(lines[1:])
    return dict(read_assignments(txt), particles=particles, basis=basis, potentials=potentials)


def read_assignments(txt):
    """method and the EXTERPOTENTIAL / INTERPOTENTIAL blocks of an input."""
    ext = [ln.split() for ln in read_block(txt, "EXTERPOTENTIAL", "END EXTERPOTENTIAL").strip().splitlines()]
    inter = [ln.split() for ln in read_block(txt, "INTERPOTENTIAL", "END INTERPOTENTIAL").strip().splitlines()]
    method = re.search(r'method\s*=\s*"([^"]+)"', txt).group(1)
    return {"method": method,
            "external": [{"species": e[0], "potential": e[1]} for e in ext if len(e) == 2],
            "inter": [{"species": [e[0], e[1]], "potential": e[2]} for e in inter if len(e) == 3]}


def potential_entries(lines, keys=None):
    """{key: components} of the 'O-<key>' entries in the lines of a potential
    (an input's POTENTIAL block or a lib/potentials file); '#' lines after the
    key are comments, as the reader skips them."""
    lines = [x.strip() for x in lines]
    entries, i = {}, 0
    while i < len(lines):
        if not lines[i].startswith("O-"):
            i += 1
            continue
        key, j = lines[i][2:], i + 1
        while lines[j].startswith("#"):
            j += 1
        n, j = int(lines[j].split()[0]), j + 1
        comps = []
        for _ in range(n):
            l = int(lines[j].split()[1])
            g, c = (float(x) for x in lines[j + 1].split()[:2])
            origin = [float(x) for x in lines[j + 2].split()[:3]]
            comps.append({"l": l, "exponent": g, "coefficient": c, "origin": origin})
            j += 3
        if keys is None or key in keys:
            entries[key] = comps
        i = j
    return entries


def read_potential_file(name, keys):
    """The given entries of lib/potentials/<name>."""
    return potential_entries(open(os.path.join(ROOT, "lib", "potentials", name)).read().splitlines(), keys)


def read_checker(name):
    txt = open(os.path.join(ROOT, "test", name)).read()
    vals = {}
    m = re.search(r"refTotalEnergy\s*=\s*([-0-9.Ee+]+)", txt)
    if m:
        vals["HF energy"] = [float(m.group(1)), 1e-8]
    m = re.search(r"refMP2Energy\s*=\s*([-0-9.Ee+]+)", txt)
    if m:
        vals["MP2 energy"] = [float(m.group(1)), 1e-5]
    for key, val, tol in re.findall(r'"([^"]+)"\s*:\s*\[\s*([-0-9.Ee+]+)\s*,\s*([-0-9.Ee+]+)\s*\]', txt):
        vals[key] = [float(val), float(tol)]
    return vals


def main():
    data = {
        "source": "generated by tests/golden/make_golden.py from the openLOWDIN tree",
        "basis": {
            "6-311G:H": read_basis("6-311G", "HYDROGEN", "H"),
            "6-311G:O": read_basis("6-311G", "OXYGEN", "O"),
            "NAKAI-5-SPD:H_1": read_basis("NAKAI-5-SPD", "HYDROGEN_1", "H_1"),
            "CC-PVDZ:H": read_basis("CC-PVDZ", "HYDROGEN", "H"),
            "CC-PVDZ:O": read_basis("CC-PVDZ", "OXYGEN", "O"),
            "6-31G.D.P:H": read_basis("6-31G.D.P", "HYDROGEN", "H"),
            "DZSNB:H_1": read_basis("DZSNB", "HYDROGEN", "H_1"),
            "DZSPNB:H_1": read_basis("DZSPNB", "HYDROGEN", "H_1"),
            "DZSPDN:H_1": read_basis("DZSPDN", "HYDROGEN", "H_1"),
            "CC-PVTZ:F": read_basis("CC-PVTZ", "FLUORINE", "F"),
            "CC-PVTZ:H": read_basis("CC-PVTZ", "HYDROGEN", "H"),
            "NAKAI-3-SPD:H_1": read_basis("NAKAI-3-SPD", "HYDROGEN_1", "H_1"),
            "NAKAI-3-SP:H_1": read_basis("NAKAI-3-SP", "HYDROGEN_1", "H_1"),
            "6-31G:H": read_basis("6-31G", "HYDROGEN", "H"),
            "6-31G:O": read_basis("6-31G", "OXYGEN", "O"),
            "6-31G:He": read_basis("6-31G", "HELIUM", "HE"),
            "6-31G.D:N": read_basis("6-31G.D", "NITROGEN", "N"),
            "6-31G.D:C": read_basis("6-31G.D", "CARBON", "C"),
            "6-31G.D:O": read_basis("6-31G.D", "OXYGEN", "O"),
            "6-311G.D.P:Ne": read_basis("6-311G.D.P", "NEON", "NE"),
            "NAKAI-7-SP:H_1": read_basis("NAKAI-7-SP", "HYDROGEN_1", "H_1"),
            "NAKAI-3-S:H_1": read_basis("NAKAI-3-S", "HYDROGEN_1", "H_1"),
            "6-31G.D:H": read_basis("6-31G.D", "HYDROGEN", "H"),
            "E+-H-7SP-AUG-CC-PVTZ:E+": read_basis("E+-H-7SP-AUG-CC-PVTZ", "POSITRON", "E+"),
            "6-311++G.D.P:H": read_basis("6-311++G.D.P", "HYDROGEN", "H"),
            "6-311++G.D.P:O": read_basis("6-311++G.D.P", "OXYGEN", "O"),
        },
        "geometry": {
            "H2O.BOA.DIRECT": read_geometry("H2O.BOA.DIRECT.lowdin"),
            "H2O.APMO.MP2": read_geometry("H2O.APMO.MP2.lowdin"),
            "HOO+.ROCI-HF": read_geometry("HOO+.ROCI-HF.lowdin"),
            "H3+.FCI": read_geometry("H3+.FCI.lowdin"),
            "H.APMO.READCOEFF": read_geometry("H.APMO.READCOEFF.lowdin"),
            "HF.APMO": read_geometry("HF.APMO.lowdin"),
            "H2.APMO.UEN": read_geometry("H2.APMO.UEN.lowdin"),
            "H2O.BOA.UEN": read_geometry("H2O.BOA.UEN.lowdin"),
            "H2O.APMO.iter0": read_geometry("H2O.APMO.iter0.lowdin"),
            "NH3.APMO.convBoth": read_geometry("NH3.APMO.convBoth.lowdin"),
            "PsH.P3": read_geometry("PsH.P3.lowdin"),
            "H2O.APMO.UP2": read_geometry("H2O.APMO.UP2.lowdin"),
            "H2O.APMO.FCI": read_geometry("H2O.APMO.FCI.lowdin"),
            "CO.CISD-dipole": read_geometry("CO.CISD-dipole.lowdin"),
            "Ne.CISD": read_geometry("Ne.CISD.lowdin"),
            "H2O.BOA": read_geometry("H2O.BOA.lowdin"),
            "H2O.BOA.UMP2": read_geometry("H2O.BOA.UMP2.lowdin"),
            "He.POTENTIALS": read_geometry("He.POTENTIALS.lowdin"),
        },
        "values": {
            "H2O.BOA.DIRECT": read_checker("H2O.BOA.DIRECT.py"),
            "H2O.BOA.MP2.DIRECT": read_checker("H2O.BOA.MP2.DIRECT.py"),
            "H2O.APMO.MP2": read_checker("H2O.APMO.MP2.py"),
            "H2O.APMO.UHF.DIRECT": read_checker("H2O.APMO.UHF.DIRECT.py"),
            "H2O.APMO.UMP2.DIRECT": read_checker("H2O.APMO.UMP2.DIRECT.py"),
            "HOO+.ROCI-HF": read_checker("HOO+.ROCI-HF.py"),
            "H3+.FCI": read_checker("H3+.FCI.py"),
            "H.APMO.READCOEFF": read_checker("H.APMO.READCOEFF.py"),
            "HF.APMO": read_checker("HF.APMO.py"),
            "H2.APMO.UEN": read_checker("H2.APMO.UEN.py"),
            "H2O.BOA.UEN": read_checker("H2O.BOA.UEN.py"),
            "H2O.APMO.iter0": read_checker("H2O.APMO.iter0.py"),
            "H2O.APMO.iter1": read_checker("H2O.APMO.iter1.py"),
            "H2O.APMO.iter2": read_checker("H2O.APMO.iter2.py"),
            "H2O.APMO.iter3": read_checker("H2O.APMO.iter3.py"),
            "NH3.APMO.convBoth": read_checker("NH3.APMO.convBoth.py"),
            "NH3.APMO.convDens": read_checker("NH3.APMO.convDens.py"),
            "NH3.APMO.convEne": read_checker("NH3.APMO.convEne.py"),
            "PsH.P3": read_checker("PsH.P3.py"),
            "H2O.APMO.UP2": read_checker("H2O.APMO.UP2.py"),
            "H2O.APMO.FCI": read_checker("H2O.APMO.FCI.py"),
            "CO.CISD-dipole": read_checker("CO.CISD-dipole.py"),
            "Ne.CISD": read_checker("Ne.CISD.py"),
            "H2O.BOA": read_checker("H2O.BOA.py"),
            "H2O.BOA.UMP2": read_checker("H2O.BOA.UMP2.py"),
            "He.POTENTIALS": read_checker("He.POTENTIALS.py"),
            "He2-C60potential-NOCI": read_checker("He2-C60potential-NOCI.py"),
            "He3-C60potential-NOCI": read_checker("He3-C60potential-NOCI.py"),
            "TIP4P-dimer-singlet-direct": read_checker("TIP4P-dimer-singlet-direct.py"),
            "TIP4P-dimer-triplet-direct": read_checker("TIP4P-dimer-triplet-direct.py"),
        },
        "g12_inputs": {
            "TIP4P-dimer-singlet-direct": read_g12_input("TIP4P-dimer-singlet-direct"),
            "TIP4P-dimer-triplet-direct": read_g12_input("TIP4P-dimer-triplet-direct"),
            "He2-C60potential-NOCI": read_c60_input("He2-C60potential-NOCI"),
            "He3-C60potential-NOCI": read_c60_input("He3-C60potential-NOCI"),
            "He.POTENTIALS": dict(read_assignments(open(os.path.join(ROOT, "test", "He.POTENTIALS.lowdin")).read()),
                                  potentials={"HEE": read_potential_file("HEE", ("E-ALPHA", "E-BETA")),
                                              "EE": read_potential_file("EE", ("E-ALPHAE-ALPHA", "E-ALPHAE-BETA",
                                                                               "E-BETAE-BETA"))}),
        },
    }
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
